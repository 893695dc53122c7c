// jv_kernels.cuh -- device code shared by the fftm kernels: complex helpers,
// the small-DFT codelets, view addressing, and the two general kernels
//
//   k_smem : a whole transform (or several) per CTA, resident in shared
//            memory; self-sorting (Stockham) radix passes with the codelets
//            2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16,
//            each thread holding its butterflies in registers across the
//            pass; R2C packing/Hermitian split and C2R un-split are fused into
//            the load and store phases.
//   k_gpass: one radix pass over every transform, global memory to global
//            memory (lengths that do not fit shared memory, or that have a
//            prime factor above 7).
//
// Both compute forward transforms; the inverse runs as conj(F(conj(x))) with
// the conjugations folded into the load and store of each element.
#pragma once

#include <cuda.h>  // CUtensorMap
#include <cuda_runtime.h>
#include <stdint.h>

#include "jv_tc.cuh"

#include "jv_core.h"

namespace jv {

template <typename T> struct cplx_t;
template <> struct cplx_t<float> { typedef float2 t; };
template <> struct cplx_t<double> { typedef double2 t; };

template <typename C> __device__ __forceinline__ C mk(decltype(C::x) a, decltype(C::x) b) {
    C r;
    r.x = a;
    r.y = b;
    return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return mk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return mk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return mk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C> __device__ __forceinline__ C cscale(C a, decltype(C::x) s) { return mk<C>(a.x * s, a.y * s); }
// multiply by -i
template <typename C> __device__ __forceinline__ C mul_mi(C a) { return mk<C>(a.y, -a.x); }
template <typename C> __device__ __forceinline__ C cconj(C a) { return mk<C>(a.x, -a.y); }

// ---------------------------------------------------------------- codelets (forward DFTs)
// In place on v[0..R-1]: v_k <- sum_n v_n exp(-2 pi i nk/R).
template <typename C, int R> struct Dft;

template <typename C> struct Dft<C, 2> {
    static __device__ __forceinline__ void run(C *v) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <typename C> struct Dft<C, 4> {
    static __device__ __forceinline__ void run(C *v) {
        C s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        C s13 = cadd(v[1], v[3]), d13 = mul_mi(csub(v[1], v[3]));
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = cadd(d02, d13);
        v[3] = csub(d02, d13);
    }
};

template <typename C> struct Dft<C, 8> {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        const T h = (T)0.707106781186547524400844362104849039;
        C e[4] = {v[0], v[2], v[4], v[6]};
        C o[4] = {v[1], v[3], v[5], v[7]};
        Dft<C, 4>::run(e);
        Dft<C, 4>::run(o);
        // twiddles exp(-2 pi i k/8), k = 1,2,3
        C o1 = mk<C>(h * (o[1].x + o[1].y), h * (o[1].y - o[1].x));
        C o2 = mul_mi(o[2]);
        C o3 = mk<C>(h * (o[3].y - o[3].x), -h * (o[3].x + o[3].y));
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    }
};

template <typename C> struct Dft<C, 16> {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        // 4 x 4: columns n1 (stride 4), then twiddle exp(-2 pi i n1 k2/16), then rows
        const T c1 = (T)0.923879532511286756128183189396788933;  // cos(pi/8)
        const T s1 = (T)0.382683432365089771728459984030398866;  // sin(pi/8)
        const T h = (T)0.707106781186547524400844362104849039;
        C a[4][4];
#pragma unroll
        for (int n1 = 0; n1 < 4; n1++) {
            C t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
            Dft<C, 4>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < 4; k2++) a[n1][k2] = t[k2];
        }
        // twiddles w16^(n1*k2)
        // n1 = 1: w^0, w^1, w^2, w^3 ; n1 = 2: w^0, w^2, w^4, w^6 ; n1 = 3: w^0, w^3, w^6, w^9
        a[1][1] = cmul(a[1][1], mk<C>(c1, -s1));
        a[1][2] = mk<C>(h * (a[1][2].x + a[1][2].y), h * (a[1][2].y - a[1][2].x));
        a[1][3] = cmul(a[1][3], mk<C>(s1, -c1));
        a[2][1] = mk<C>(h * (a[2][1].x + a[2][1].y), h * (a[2][1].y - a[2][1].x));
        a[2][2] = mul_mi(a[2][2]);
        a[2][3] = mk<C>(h * (a[2][3].y - a[2][3].x), -h * (a[2][3].x + a[2][3].y));
        a[3][1] = cmul(a[3][1], mk<C>(s1, -c1));
        a[3][2] = mk<C>(h * (a[3][2].y - a[3][2].x), -h * (a[3][2].x + a[3][2].y));
        a[3][3] = cmul(a[3][3], mk<C>(-c1, s1));
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) {
            C t[4] = {a[0][k2], a[1][k2], a[2][k2], a[3][k2]};
            Dft<C, 4>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < 4; k1++) v[k2 + 4 * k1] = t[k1];
        }
    }
};

template <typename C> struct Dft<C, 3> {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        const T s3 = (T)0.866025403784438646763723170752936183;  // sin(2 pi/3)
        C s = cadd(v[1], v[2]);
        C d = csub(v[1], v[2]);
        C t = mk<C>(v[0].x - (T)0.5 * s.x, v[0].y - (T)0.5 * s.y);
        C m = mk<C>(s3 * d.y, -s3 * d.x);  // -i sin(2pi/3) d
        v[0] = cadd(v[0], s);
        v[1] = cadd(t, m);
        v[2] = csub(t, m);
    }
};

template <typename C> struct Dft<C, 5> {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        const T c1 = (T)0.309016994374947424102293417182819059;   // cos(2pi/5)
        const T c2 = (T)-0.809016994374947424102293417182819059;  // cos(4pi/5)
        const T s1 = (T)0.951056516295153572116439333379382143;   // sin(2pi/5)
        const T s2 = (T)0.587785252292473129168705954639072769;   // sin(4pi/5)
        C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        C a0 = v[0];
        C b1 = mk<C>(a0.x + c1 * t1.x + c2 * t2.x, a0.y + c1 * t1.y + c2 * t2.y);
        C b2 = mk<C>(a0.x + c2 * t1.x + c1 * t2.x, a0.y + c2 * t1.y + c1 * t2.y);
        C d1 = mk<C>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
        C d2 = mk<C>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
        v[0] = cadd(a0, cadd(t1, t2));
        // y = b -+ i d
        v[1] = mk<C>(b1.x + d1.y, b1.y - d1.x);
        v[4] = mk<C>(b1.x - d1.y, b1.y + d1.x);
        v[2] = mk<C>(b2.x + d2.y, b2.y - d2.x);
        v[3] = mk<C>(b2.x - d2.y, b2.y + d2.x);
    }
};

template <typename C> struct Dft<C, 7> {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        const T c1 = (T)0.623489801858733530525004884004239811;   // cos(2pi/7)
        const T c2 = (T)-0.222520933956314404288902564496794759;  // cos(4pi/7)
        const T c3 = (T)-0.900968867902419126236102319507445051;  // cos(6pi/7)
        const T s1 = (T)0.781831482468029808708444526674057751;   // sin(2pi/7)
        const T s2 = (T)0.974927912181823607018131682993931217;   // sin(4pi/7)
        const T s3 = (T)0.433883739117558120475768332848358755;   // sin(6pi/7)
        C a0 = v[0];
        C p1 = cadd(v[1], v[6]), m1 = csub(v[1], v[6]);
        C p2 = cadd(v[2], v[5]), m2 = csub(v[2], v[5]);
        C p3 = cadd(v[3], v[4]), m3 = csub(v[3], v[4]);
        C b1 = mk<C>(a0.x + c1 * p1.x + c2 * p2.x + c3 * p3.x, a0.y + c1 * p1.y + c2 * p2.y + c3 * p3.y);
        C b2 = mk<C>(a0.x + c2 * p1.x + c3 * p2.x + c1 * p3.x, a0.y + c2 * p1.y + c3 * p2.y + c1 * p3.y);
        C b3 = mk<C>(a0.x + c3 * p1.x + c1 * p2.x + c2 * p3.x, a0.y + c3 * p1.y + c1 * p2.y + c2 * p3.y);
        C d1 = mk<C>(s1 * m1.x + s2 * m2.x + s3 * m3.x, s1 * m1.y + s2 * m2.y + s3 * m3.y);
        C d2 = mk<C>(s2 * m1.x - s3 * m2.x - s1 * m3.x, s2 * m1.y - s3 * m2.y - s1 * m3.y);
        C d3 = mk<C>(s3 * m1.x - s1 * m2.x + s2 * m3.x, s3 * m1.y - s1 * m2.y + s2 * m3.y);
        v[0] = cadd(a0, cadd(p1, cadd(p2, p3)));
        v[1] = mk<C>(b1.x + d1.y, b1.y - d1.x);
        v[6] = mk<C>(b1.x - d1.y, b1.y + d1.x);
        v[2] = mk<C>(b2.x + d2.y, b2.y - d2.x);
        v[5] = mk<C>(b2.x - d2.y, b2.y + d2.x);
        v[3] = mk<C>(b3.x + d3.y, b3.y - d3.x);
        v[4] = mk<C>(b3.x - d3.y, b3.y + d3.x);
    }
};

// ---- composite codelets R = P*Q (6, 9, 10, 12, 14, 15) from the prime-power
// ones, with their internal twiddles exp(-2 pi i e/R) evaluated by the compiler
// (Taylor series on an exactly reduced angle, |x| <= pi/4, in double).
namespace cx {
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double sin_small(double x) {
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; k++) {
        term *= -x2 / ((2.0 * k) * (2.0 * k + 1.0));
        sum += term;
    }
    return sum;
}
constexpr double cos_small(double x) {
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k < 14; k++) {
        term *= -x2 / ((2.0 * k - 1.0) * (2.0 * k));
        sum += term;
    }
    return sum;
}
// cos and sin of 2 pi e/R: quadrant q = floor(4e/R), remainder r/R of a
// quarter turn, folded to an angle of at most pi/4
constexpr double root_cs(int R, int e, bool want_sin) {
    e %= R;
    const int q = (4 * e) / R, r = 4 * e - q * R;
    const bool fold = 2 * r > R;
    const double x = (kPi / 2.0) * (double)(fold ? R - r : r) / (double)R;
    double c = fold ? sin_small(x) : cos_small(x), s = fold ? cos_small(x) : sin_small(x);
    double cq = c, sq = s;  // rotate by q quarter turns
    if (q == 1) { cq = -s; sq = c; }
    if (q == 2) { cq = -c; sq = -s; }
    if (q == 3) { cq = s; sq = -c; }
    return want_sin ? sq : cq;
}
}  // namespace cx

template <int R, int E> struct Root {  // exp(-2 pi i E/R)
    static constexpr double c = cx::root_cs(R, E, false);
    static constexpr double s = -cx::root_cs(R, E, true);
};

template <typename C, int R, int E>
__device__ __forceinline__ C cmul_root(C a) {
    typedef decltype(C::x) T;
    const T c = (T)Root<R, E>::c, s = (T)Root<R, E>::s;
    return mk<C>(a.x * c - a.y * s, a.x * s + a.y * c);
}

// a[n2][k1] *= exp(-2 pi i n2 k1/R) for every index I = n2*P + k1 >= I0
template <typename C, int R, int P, int Q, int I>
struct PQTwiddle {
    static __device__ __forceinline__ void run(C (&a)[Q][P]) {
        constexpr int n2 = I / P, k1 = I % P;
        if constexpr (n2 * k1 != 0) a[n2][k1] = cmul_root<C, R, n2 * k1>(a[n2][k1]);
        if constexpr (I + 1 < P * Q) PQTwiddle<C, R, P, Q, I + 1>::run(a);
    }
};

// R = P*Q points: n = Q n1 + n2, k = k1 + P k2;
// X[k1 + P k2] = sum_n2 w_Q^(n2 k2) w_R^(n2 k1) sum_n1 x[Q n1 + n2] w_P^(n1 k1)
template <typename C, int P, int Q> struct DftPQ {
    static __device__ __forceinline__ void run(C *v) {
        C a[Q][P];
#pragma unroll
        for (int n2 = 0; n2 < Q; n2++) {
            C t[P];
#pragma unroll
            for (int n1 = 0; n1 < P; n1++) t[n1] = v[Q * n1 + n2];
            Dft<C, P>::run(t);
#pragma unroll
            for (int k1 = 0; k1 < P; k1++) a[n2][k1] = t[k1];
        }
        PQTwiddle<C, P * Q, P, Q, 0>::run(a);
#pragma unroll
        for (int k1 = 0; k1 < P; k1++) {
            C t[Q];
#pragma unroll
            for (int n2 = 0; n2 < Q; n2++) t[n2] = a[n2][k1];
            Dft<C, Q>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < Q; k2++) v[k1 + P * k2] = t[k2];
        }
    }
};
template <typename C> struct Dft<C, 6> : DftPQ<C, 2, 3> {};
template <typename C> struct Dft<C, 9> : DftPQ<C, 3, 3> {};
template <typename C> struct Dft<C, 10> : DftPQ<C, 2, 5> {};
template <typename C> struct Dft<C, 12> : DftPQ<C, 4, 3> {};
template <typename C> struct Dft<C, 14> : DftPQ<C, 2, 7> {};
template <typename C> struct Dft<C, 15> : DftPQ<C, 3, 5> {};

// cos and sin of 2 pi i / R (i = 1 .. (R - 1) / 2) for the odd-prime codelets:
// constants that the unrolled loops fold into their multiply-adds
template <int R> __host__ __device__ constexpr double prime_cos(int i);
template <int R> __host__ __device__ constexpr double prime_sin(int i);
template <> __host__ __device__ constexpr double prime_cos<11>(int i) {
    return i == 1 ? 0.8412535328311812
         : i == 2 ? 0.41541501300188644
         : i == 3 ? -0.142314838273285
         : i == 4 ? -0.654860733945285
         : -0.9594929736144974;
}
template <> __host__ __device__ constexpr double prime_sin<11>(int i) {
    return i == 1 ? 0.5406408174555976
         : i == 2 ? 0.9096319953545183
         : i == 3 ? 0.9898214418809328
         : i == 4 ? 0.7557495743542583
         : 0.28173255684142967;
}
template <> __host__ __device__ constexpr double prime_cos<13>(int i) {
    return i == 1 ? 0.8854560256532099
         : i == 2 ? 0.5680647467311559
         : i == 3 ? 0.120536680255323
         : i == 4 ? -0.35460488704253545
         : i == 5 ? -0.7485107481711012
         : -0.970941817426052;
}
template <> __host__ __device__ constexpr double prime_sin<13>(int i) {
    return i == 1 ? 0.4647231720437685
         : i == 2 ? 0.8229838658936564
         : i == 3 ? 0.992708874098054
         : i == 4 ? 0.9350162426854148
         : i == 5 ? 0.6631226582407952
         : 0.23931566428755768;
}
template <> __host__ __device__ constexpr double prime_cos<17>(int i) {
    return i == 1 ? 0.9324722294043558
         : i == 2 ? 0.7390089172206591
         : i == 3 ? 0.4457383557765383
         : i == 4 ? 0.09226835946330202
         : i == 5 ? -0.2736629900720829
         : i == 6 ? -0.6026346363792563
         : i == 7 ? -0.850217135729614
         : -0.9829730996839018;
}
template <> __host__ __device__ constexpr double prime_sin<17>(int i) {
    return i == 1 ? 0.3612416661871529
         : i == 2 ? 0.6736956436465572
         : i == 3 ? 0.8951632913550623
         : i == 4 ? 0.9957341762950345
         : i == 5 ? 0.961825643172819
         : i == 6 ? 0.7980172272802396
         : i == 7 ? 0.5264321628773561
         : 0.18374951781657037;
}
template <> __host__ __device__ constexpr double prime_cos<19>(int i) {
    return i == 1 ? 0.9458172417006346
         : i == 2 ? 0.7891405093963936
         : i == 3 ? 0.5469481581224269
         : i == 4 ? 0.24548548714079924
         : i == 5 ? -0.08257934547233227
         : i == 6 ? -0.4016954246529694
         : i == 7 ? -0.6772815716257409
         : i == 8 ? -0.879473751206489
         : -0.9863613034027223;
}
template <> __host__ __device__ constexpr double prime_sin<19>(int i) {
    return i == 1 ? 0.32469946920468346
         : i == 2 ? 0.6142127126896678
         : i == 3 ? 0.8371664782625285
         : i == 4 ? 0.9694002659393304
         : i == 5 ? 0.9965844930066698
         : i == 6 ? 0.9157733266550574
         : i == 7 ? 0.7357239106731318
         : i == 8 ? 0.4759473930370737
         : 0.16459459028073403;
}
template <> __host__ __device__ constexpr double prime_cos<23>(int i) {
    return i == 1 ? 0.9629172873477992
         : i == 2 ? 0.8544194045464886
         : i == 3 ? 0.6825531432186541
         : i == 4 ? 0.4600650377311522
         : i == 5 ? 0.20345601305263375
         : i == 6 ? -0.06824241336467088
         : i == 7 ? -0.33487961217098616
         : i == 8 ? -0.5766803221148671
         : i == 9 ? -0.7757112907044197
         : i == 10 ? -0.917211301505453
         : -0.9906859460363306;
}
template <> __host__ __device__ constexpr double prime_sin<23>(int i) {
    return i == 1 ? 0.2697967711570243
         : i == 2 ? 0.5195839500354336
         : i == 3 ? 0.730835964278124
         : i == 4 ? 0.8878852184023752
         : i == 5 ? 0.9790840876823229
         : i == 6 ? 0.9976687691905392
         : i == 7 ? 0.9422609221188205
         : i == 8 ? 0.8169698930104421
         : i == 9 ? 0.631087944326053
         : i == 10 ? 0.3984010898462414
         : 0.1361666490962471;
}

// Odd prime R as a direct O(R^2) DFT in registers, halved by the symmetry of
// the roots: with s_n = v_n + v_(R-n) and d_n = v_n - v_(R-n) (n = 1 .. H,
// H = (R - 1) / 2), Y_0 = v_0 + sum s_n and, for k = 1 .. H,
// Y_k = a_k - i b_k, Y_(R-k) = a_k + i b_k, a_k = v_0 + sum s_n cos(2 pi nk/R),
// b_k = sum d_n sin(2 pi nk/R) -- the forward DFT of VI_dftm_f
// (c_VSIP_src/VI_fftm_building_blocks_f.h:95-155) for one butterfly.
template <typename C, int R> struct DftOdd {
    static __device__ __forceinline__ void run(C *v) {
        typedef decltype(C::x) T;
        constexpr int H = (R - 1) / 2;
        C s[H], d[H];
        C y0 = v[0];
#pragma unroll
        for (int n = 1; n <= H; n++) {
            s[n - 1] = cadd(v[n], v[R - n]);
            d[n - 1] = csub(v[n], v[R - n]);
            y0 = cadd(y0, s[n - 1]);
        }
        C y[R];
        y[0] = y0;
#pragma unroll
        for (int k = 1; k <= H; k++) {
            C a = v[0], b = mk<C>((T)0, (T)0);
#pragma unroll
            for (int n = 1; n <= H; n++) {
                // 2 pi nk/R reduced to i = nk mod R, folded into 1 .. H (sin changes sign)
                const int e = (n * k) % R;
                const int i = e <= H ? e : R - e;
                const T c = (T)prime_cos<R>(i), sn = (T)(e <= H ? prime_sin<R>(i) : -prime_sin<R>(i));
                a.x += s[n - 1].x * c;
                a.y += s[n - 1].y * c;
                b.x += d[n - 1].x * sn;
                b.y += d[n - 1].y * sn;
            }
            y[k] = mk<C>(a.x + b.y, a.y - b.x);
            y[R - k] = mk<C>(a.x - b.y, a.y + b.x);
        }
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = y[r];
    }
};
template <typename C> struct Dft<C, 11> : DftOdd<C, 11> {};
template <typename C> struct Dft<C, 13> : DftOdd<C, 13> {};
template <typename C> struct Dft<C, 17> : DftOdd<C, 17> {};
template <typename C> struct Dft<C, 19> : DftOdd<C, 19> {};
template <typename C> struct Dft<C, 23> : DftOdd<C, 23> {};

// ---------------------------------------------------------------- view access
// Complex element (v, n) of a CView; `conj` negates the imaginary part.
template <typename T> struct CAcc {
    typedef typename cplx_t<T>::t C;
    const T *re, *im;
    long cst, off, es, vs;
    bool vec;  // interleaved and aligned: one vector load per element
    __device__ __forceinline__ long idx(long v, long n) const { return cst * (off + v * vs + n * es); }
    __device__ __forceinline__ C load(long v, long n) const {
        long i = idx(v, n);
        if (vec) return *reinterpret_cast<const C *>(re + i);
        return mk<C>(re[i], im[i]);
    }
    // element at complex index g (= off + v*vs + n*es)
    __device__ __forceinline__ C at(long g) const {
        if (vec) return reinterpret_cast<const C *>(re)[g];
        return mk<C>(re[cst * g], im[cst * g]);
    }
};
template <typename T> struct CSto {
    typedef typename cplx_t<T>::t C;
    T *re, *im;
    long cst, off, es, vs;
    bool vec;
    __device__ __forceinline__ long idx(long v, long n) const { return cst * (off + v * vs + n * es); }
    __device__ __forceinline__ void store(long v, long n, C c) const {
        long i = idx(v, n);
        if (vec) {
            *reinterpret_cast<C *>(re + i) = c;
        } else {
            re[i] = c.x;
            im[i] = c.y;
        }
    }
    __device__ __forceinline__ void put(long g, C c) const {
        if (vec) {
            reinterpret_cast<C *>(re)[g] = c;
        } else {
            re[cst * g] = c.x;
            im[cst * g] = c.y;
        }
    }
};
template <typename T> struct RAcc {
    const T *a;
    long rst, off, es, vs;
    __device__ __forceinline__ T load(long v, long n) const { return a[rst * (off + v * vs + n * es)]; }
};
template <typename T> struct RSto {
    T *a;
    long rst, off, es, vs;
    __device__ __forceinline__ void store(long v, long n, T x) const { a[rst * (off + v * vs + n * es)] = x; }
};

// floor(x / d) by a multiply-high with m = ceil(2^32 / d), exact whenever
// x * d < 2^32 (every index of one CTA's tile: x, d < 2^16); m = 0 encodes d = 1
__device__ __forceinline__ unsigned magic_of(unsigned d) { return d <= 1 ? 0u : 0xFFFFFFFFu / d + 1u; }
__device__ __forceinline__ int mdiv(int x, unsigned m) { return m ? (int)__umulhi((unsigned)x, m) : x; }

// Walker constants computed at launch for a grid of width B and blockDim threads.
struct WalkConst {
    int B, da, db;
    unsigned mB;
};
inline WalkConst walk_const(long B, long nthr) {
    WalkConst c;
    c.B = (int)B;
    c.da = (int)(nthr / B);
    c.db = (int)(nthr % B);
    c.mB = magic_host((unsigned long)B);
    return c;
}

// Walks i = i0, i0 + step, ... over an A x B grid (i = a*B + b, b fastest)
// keeping the global element index g = g0 + a*sa + b*sb up to date with adds:
// one division per thread at the start, none per element.
struct Walk {
    int a, b, B, da, db;
    long g, dg, dgw;
    __device__ __forceinline__ void init(int i0, int step, int B_, long sa, long sb, long g0) {
        B = B_;
        a = i0 / B;
        b = i0 - a * B;
        da = step / B;
        db = step - da * B;
        g = g0 + (long)a * sa + (long)b * sb;
        dg = (long)da * sa + (long)db * sb;
        dgw = sa - (long)B * sb;
    }
    // the same from launch-time constants (B, nthr / B, nthr % B, magic of B):
    // no division at all
    __device__ __forceinline__ void init_c(const WalkConst c, long sa, long sb, long g0) {
        B = c.B;
        a = mdiv((int)threadIdx.x, c.mB);
        b = (int)threadIdx.x - a * B;
        da = c.da;
        db = c.db;
        g = g0 + (long)a * sa + (long)b * sb;
        dg = (long)da * sa + (long)db * sb;
        dgw = sa - (long)B * sb;
    }
    __device__ __forceinline__ void next() {
        a += da;
        b += db;
        g += dg;
        if (b >= B) {
            b -= B;
            a++;
            g += dgw;
        }
    }
};

// ---------------------------------------------------------------- shared-memory kernel
template <typename T> struct SmemArgs {
    typedef typename cplx_t<T>::t C;
    int kind;         // K_C2C / K_R2C / K_C2R
    int N;            // complex FFT length
    int ld;           // shared-memory row pitch (complex elements) >= N (+1 for C2R)
    int vpb;          // transforms per CTA
    long nvec;
    int inv;
    int has_scale;
    T scale;
    int vec_fast;     // global load/store mapping: consecutive threads -> consecutive transforms
    unsigned long long passes;  // pass counts per codelet (pass_count)
    const uint4 *pc;  // per-pass constants of the schedule (NR, magic NR, Ns, magic Ns)
    unsigned mvpb;    // multiply-high magic of vpb
    int real_pairs;   // R2C input / C2R output rows: unit stride, even offset and pitch, 2-element aligned
    // column tiles of c2c loaded by TMA: boxes of (2*vpb scalars) x tma_rows
    // rows of the input view (tmap), tma_boxes per tile, tma_bytes in all
    int tma, tma_boxes, tma_rows;
    unsigned tma_bytes;
    // test hook (jvsip_gpu_test_wait_expiry): after the boxes have landed,
    // wait on the barrier's next phase, which nothing completes, so the
    // bounded wait runs out with no copy in flight
    int tma_expire;
    int *status;      // set to 1 when the bounded wait for the boxes expired
    // c2c tiles of column-type views: ld_rows / st_rows load / store with
    // consecutive threads on consecutive elements of one transform (the view
    // side that is row-contiguous), the other side with consecutive threads on
    // adjacent transforms
    int ld_rows, st_rows;
    int conj_in, conj_out;  // conjugate on load / on store (both = inv for a whole transform)
    // batch of vector groups along gridDim.y: group y starts bvs_in / bvs_out
    // complex elements after group 0 (the steps of a long transform)
    long bvs_in, bvs_out;
    // output twiddle of the first step of a long transform: output element k
    // of transform t in group y is multiplied by W^(g*k), g = t*tw_ts +
    // (y0 + y)*tw_ys, as tw_lo[m & tw_mask] * tw_hi[m >> tw_sh], m = g*k
    const typename cplx_t<T>::t *tw_lo, *tw_hi;
    unsigned tw_mask, tw_sh, tw_ts, tw_ys;
    long y0;          // group index of this launch's first group
    // the k-omega pipeline's fused prologue / epilogue (instances KX_R2C_TAPER,
    // KX_C2C_POWER only): real element n of transform t is multiplied by
    // tp_n[n*tp_n_st] and then by tp_t[t*tp_t_st] as it is loaded (and written
    // back when tp_back); output element k of transform t stores
    // (g_scale*|X|^2, Im X) and adds g_scale*|X|^2 to gram[t*g_vs + k*g_es]
    const T *tp_n, *tp_t;
    long tp_n_st, tp_t_st;
    int tp_back;
    T *gram;
    long g_es, g_vs;
    T g_scale;
    CUtensorMap tmap;
    WalkConst win, wout;  // load / store walker constants for full tiles of vpb transforms
    CAcc<T> cin;
    CSto<T> cout;
    RAcc<T> rin;
    RSto<T> rout;
    const C *tw;      // exp(-2 pi i m/N)
    const C *twg;     // per-pass tables of the radix schedule, [r][m] each
    const C *thalf;   // exp(-+ i pi k/N), k <= N
};

// One in-place radix-R pass over the CTA's transforms in shared memory.
// Butterfly b of transform t reads elements j + r*N/R and writes
// (j - m)*R + m + r*Ns, m = j mod Ns, after the twiddle exp(-2 pi i r m/(Ns R)).
// A thread keeps all its butterflies in registers across the barrier, so the
// pass needs ceil(EMAX/R) * blockDim >= transforms * N/R.
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }

// pass counts per codelet (order of kRadixList), 4 bits each
__host__ __device__ __forceinline__ int pass_count(unsigned long long packed, int i) {
    return (int)((packed >> (4 * i)) & 15ull);
}

template <typename T, int R, int EMAX, int IN = 0>
__device__ __forceinline__ void smem_pass(typename cplx_t<T>::t *s, int ld, int nt, int Ns,
                                          const typename cplx_t<T>::t *__restrict__ tp, const uint4 pc, int dp = 0) {
    // IN: where the pass reads -- 0 the padded rows; 1 dense rows (t*ld + n);
    // 2 dense transposed (n*dp + t), the order a TMA box of adjacent
    // transforms lands in (the first pass over data that arrived in natural
    // order; the pass writes the padded rows in place)
    // tp: this pass's twiddles, entry r*Ns + m = exp(-2 pi i r m/(Ns R)), so the
    // threads of a warp (consecutive m) read consecutive entries; pc: NR = N/R,
    // the multiply-high magic numbers of NR and Ns
    typedef typename cplx_t<T>::t C;
    constexpr int K = pass_k(EMAX, R);
    const int NR = (int)pc.x;
    const int nb = nt * NR;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const unsigned mNR = pc.y, mNs = pc.w;
    C v[K][R];
#pragma unroll
    for (int k = 0; k < K; k++) {
        int b = tid + k * nthr;
        if (b < nb) {
            int t = mdiv(b, mNR), j = b - t * NR;
            const C *src = s + t * ld;
#pragma unroll
            for (int r = 0; r < R; r++)
                v[k][r] = (IN == 2) ? s[(j + r * NR) * dp + t] : src[IN == 1 ? (j + r * NR) : spad(j + r * NR)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
        int b = tid + k * nthr;
        if (b < nb) {
            int t = mdiv(b, mNR), j = b - t * NR;
            int m = (Ns == 1) ? 0 : j - Ns * mdiv(j, mNs);
            if (m) {
#pragma unroll
                for (int r = 1; r < R; r++) v[k][r] = cmul(v[k][r], __ldg(&tp[r * Ns + m]));
            }
            Dft<C, R>::run(v[k]);
            C *dst = s + t * ld;
            const int base = (j - m) * R + m;
#pragma unroll
            for (int r = 0; r < R; r++) dst[spad(base + r * Ns)] = v[k][r];
        }
    }
    __syncthreads();
}

// The plan's schedule: `packed` pass counts per codelet in the order of
// kRadixList (the order of the plan's per-pass twiddle tables twg and pass
// constants pc).  One loop per codelet keeps the codelets' register lifetimes
// apart.
template <typename T, int EMAX>
__device__ __forceinline__ void smem_passes_from(typename cplx_t<T>::t *s, int ld, int nt, unsigned long long packed,
                                                 const typename cplx_t<T>::t *__restrict__ &tp,
                                                 const uint4 *__restrict__ pc, int &Ns, int &p);

template <typename T, int EMAX>
__device__ __forceinline__ void smem_passes(typename cplx_t<T>::t *s, int ld, int nt, unsigned long long packed,
                                            const typename cplx_t<T>::t *__restrict__ twg,
                                            const uint4 *__restrict__ pc) {
    int Ns = 1, p = 0;
    const typename cplx_t<T>::t *tp = twg;
    smem_passes_from<T, EMAX>(s, ld, nt, packed, tp, pc, Ns, p);
}

// ---------------------------------------------------------------- fused first / last passes (c2c)
// A c2c tile's first radix pass reads the view in global memory directly and
// its last pass writes the view directly, so a tile crosses shared memory only
// between passes.  Butterfly b of the tile maps to (transform t, index j):
// j fastest for row tiles (consecutive threads read consecutive elements),
// t fastest for column tiles (consecutive threads read adjacent transforms).
// x with its sign bit flipped when m = 0x80000000 (exact negation on the
// integer pipe; m = 0 leaves x unchanged)
__device__ __forceinline__ float flip_sign(float x, unsigned m) { return __int_as_float(__float_as_int(x) ^ (int)m); }
__device__ __forceinline__ double flip_sign(double x, unsigned m) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)m << 32));
}

// the stored value: conjugated back for the inverse, scaled when the plan has a
// scale (single precision multiplies by 1 otherwise, which is exact; double
// precision, bound by its FP64 pipe, skips the multiply)
template <typename C, typename T>
__device__ __forceinline__ C out_value(C v, unsigned smask, bool has_scale, T scale) {
    v.y = flip_sign(v.y, smask);
    if (sizeof(T) == 4 || has_scale) {
        v.x *= scale;
        v.y *= scale;
    }
    return v;
}

// single roundings without contraction into fused multiply-adds
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T> struct TileIO {
    typedef typename cplx_t<T>::t C;
    const C *in;     // interleaved input; element (t, n) at in[t*in_vs + n*in_es]
    C *out;          // interleaved output; element (t, n) at out[t*out_vs + n*out_es]
    long in_es, in_vs, out_es, out_vs;
    unsigned smask_in, smask_out;  // 0x80000000: conjugate on load / on store, else 0
    bool has_scale;
    T scale;         // 1 when the plan has no scale
    bool vf;         // t-fastest mapping of the loads
    bool vf_out;     // t-fastest mapping of the stores
    unsigned mnt;    // multiply-high magic of the tile's transform count
    // output twiddle W^(g*k), g = tw_t0 + t*tw_ts (none when tw_lo is null)
    const C *tw_lo, *tw_hi;
    unsigned tw_mask, tw_sh, tw_t0, tw_ts;
    // fused prologue / epilogue of the k-omega pipeline (FX template flag of
    // the passes): tapers of the loaded real pairs (element and transform),
    // the write-back target of the tapered input, and the power accumulator
    const T *tp_n, *tp_t;
    long tp_n_st, tp_t_st;
    C *wb;
    T *gram;
    long g_es, g_vs;
    T g_scale;
    // split complex views (FX_SPLIT): element (t, n) at in_re / in_im
    // [t*in_vs + n*in_es], out_re / out_im [t*out_vs + n*out_es]
    const T *in_re, *in_im;
    T *out_re, *out_im;
};

// FX flags of the fused passes
constexpr int FX_TAPER = 1;  // first pass: taper the loaded real pairs, optionally write them back
constexpr int FX_POWER = 2;  // last pass: store (s|X|^2, Im X), gram += s|X|^2
constexpr int FX_SPLIT = 4;  // split complex views: real and imaginary parts in separate arrays

template <int FX, typename C, typename T>
__device__ __forceinline__ C io_load(const TileIO<T> &io, const C *src, long e) {
    if constexpr ((FX & FX_SPLIT) != 0) return mk<C>(io.in_re[e], io.in_im[e]);
    else return src[e];
}
template <int FX, typename C, typename T>
__device__ __forceinline__ void io_store(const TileIO<T> &io, C *dst, long e, C v) {
    if constexpr ((FX & FX_SPLIT) != 0) {
        io.out_re[e] = v.x;
        io.out_im[e] = v.y;
    } else {
        dst[e] = v;
    }
}

// the tapered pair at complex index n of transform t: x_2n*tp_n[2n] then
// *tp_t[t] (c_VSIP_src/vsip_vmmul_f.c: rows by the time taper, then columns by
// the array taper; products rounded in that order)
template <typename C, typename T>
__device__ __forceinline__ C taper_pair(C c, const TileIO<T> &io, long n, int t) {
    const T wt = io.tp_t[(long)t * io.tp_t_st];
    const T w0 = io.tp_n[2 * n * io.tp_n_st], w1 = io.tp_n[(2 * n + 1) * io.tp_n_st];
    c.x = mul_rn(mul_rn(w0, c.x), wt);
    c.y = mul_rn(mul_rn(w1, c.y), wt);
    return c;
}

// p = |v|^2 (c_VSIP_src/vsip_mcmagsq_f.c), p *= s (vsip_smmul_f.c),
// gram = p + gram (vsip_madd_f.c), each rounded in that order; stores (p, Im v)
template <typename C, typename T>
__device__ __forceinline__ C power_out(C v, const TileIO<T> &io, long t, long k) {
    T p = add_rn(mul_rn(v.x, v.x), mul_rn(v.y, v.y));
    p = mul_rn(io.g_scale, p);
    T *g = io.gram + t * io.g_vs + k * io.g_es;
    *g = add_rn(p, *g);
    return mk<C>(p, v.y);
}

// W^m from the two-level table of a long transform's output twiddles
template <typename C>
__device__ __forceinline__ C tw_two_level(const C *__restrict__ lo, const C *__restrict__ hi, unsigned mask,
                                          unsigned sh, unsigned m) {
    return cmul(__ldg(&lo[m & mask]), __ldg(&hi[m >> sh]));
}

__device__ __forceinline__ void tile_tj(int b, bool vf, int nt, unsigned mnt, int NR, unsigned mNR, int &t, int &j) {
    if (vf) {
        j = mdiv(b, mnt);
        t = b - j * nt;
    } else {
        t = mdiv(b, mNR);
        j = b - t * NR;
    }
}

// First pass (Ns = 1, no twiddle) from global memory; to shared memory, or,
// for a one-pass schedule (LAST), straight back to global memory.
template <typename T, int R, int EMAX, bool LAST, int FX = 0>
__device__ __forceinline__ void pass_first(typename cplx_t<T>::t *s, int ld, int nt, const uint4 pc,
                                           const TileIO<T> &io) {
    typedef typename cplx_t<T>::t C;
    constexpr int K = pass_k(EMAX, R);
    const int NR = (int)pc.x, nb = nt * NR;
    const int tid = threadIdx.x, nthr = blockDim.x;
    C v[K][R];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int b = tid + k * nthr;
        if (b < nb) {
            int t, j;
            tile_tj(b, io.vf, nt, io.mnt, NR, pc.y, t, j);
            const long e0 = (long)t * io.in_vs + (long)j * io.in_es;
            const long st = (long)NR * io.in_es;
#pragma unroll
            for (int r = 0; r < R; r++) {
                C c = io_load<FX>(io, io.in, e0 + r * st);
                if constexpr ((FX & FX_TAPER) != 0) {
                    c = taper_pair(c, io, (long)(j + r * NR), t);
                    if (io.wb) io.wb[(long)t * io.in_vs + (long)(j + r * NR) * io.in_es] = c;
                }
                c.y = flip_sign(c.y, io.smask_in);
                v[k][r] = c;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int b = tid + k * nthr;
        if (b < nb) {
            int t, j;
            tile_tj(b, io.vf, nt, io.mnt, NR, pc.y, t, j);
            Dft<C, R>::run(v[k]);
            if (LAST) {
                // one pass: N = R, j = 0, output element r
#pragma unroll
                for (int r = 0; r < R; r++) {
                    C o = out_value(v[k][r], io.smask_out, io.has_scale, io.scale);
                    if constexpr ((FX & FX_POWER) != 0) o = power_out(o, io, (long)t, (long)r);
                    io_store<FX>(io, io.out, (long)t * io.out_vs + r * io.out_es, o);
                }
            } else {
                C *dst = s + t * ld;
#pragma unroll
                for (int r = 0; r < R; r++) dst[spad(j * R + r)] = v[k][r];
            }
        }
    }
    if (!LAST) __syncthreads();
}

// Last pass (Ns = N/R, so m = j) from shared memory to global memory.
template <typename T, int R, int EMAX, int FX = 0>
__device__ __forceinline__ void pass_last(const typename cplx_t<T>::t *s, int ld, int nt, int Ns,
                                          const typename cplx_t<T>::t *__restrict__ tp, const uint4 pc,
                                          const TileIO<T> &io) {
    typedef typename cplx_t<T>::t C;
    constexpr int K = pass_k(EMAX, R);
    const int NR = (int)pc.x, nb = nt * NR;
    const int tid = threadIdx.x, nthr = blockDim.x;
    C v[K][R];
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int b = tid + k * nthr;
        if (b < nb) {
            int t, j;
            tile_tj(b, io.vf_out, nt, io.mnt, NR, pc.y, t, j);
            const C *src = s + t * ld;
#pragma unroll
            for (int r = 0; r < R; r++) v[k][r] = src[spad(j + r * NR)];
        }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
        const int b = tid + k * nthr;
        if (b < nb) {
            int t, j;
            tile_tj(b, io.vf_out, nt, io.mnt, NR, pc.y, t, j);
            if (j) {
#pragma unroll
                for (int r = 1; r < R; r++) v[k][r] = cmul(v[k][r], __ldg(&tp[r * Ns + j]));
            }
            Dft<C, R>::run(v[k]);
            if (io.tw_lo) {
                // output element j + r*Ns of transform t: times W^(g*(j + r*Ns))
                const unsigned tg = io.tw_t0 + (unsigned)t * io.tw_ts;
#pragma unroll
                for (int r = 0; r < R; r++)
                    v[k][r] = cmul(v[k][r], tw_two_level(io.tw_lo, io.tw_hi, io.tw_mask, io.tw_sh,
                                                         tg * (unsigned)(j + r * Ns)));
            }
            const long e0 = (long)t * io.out_vs + (long)j * io.out_es;
            const long st = (long)Ns * io.out_es;
#pragma unroll
            for (int r = 0; r < R; r++) {
                C o = out_value(v[k][r], io.smask_out, io.has_scale, io.scale);
                if constexpr ((FX & FX_POWER) != 0) o = power_out(o, io, (long)t, (long)(j + r * Ns));
                io_store<FX>(io, io.out, e0 + r * st, o);
            }
        }
    }
}

#define JV_RADIX_SWITCH(I, CALL) \
    switch (I) {                 \
        case 0: CALL(16); break; \
        case 1: CALL(15); break; \
        case 2: CALL(14); break; \
        case 3: CALL(12); break; \
        case 4: CALL(10); break; \
        case 5: CALL(9); break;  \
        case 6: CALL(8); break;  \
        case 7: CALL(7); break;  \
        case 8: CALL(6); break;  \
        case 9: CALL(5); break;  \
        case 10: CALL(4); break; \
        case 11: CALL(3); break; \
        default: CALL(2); break; \
    }

// The passes of a tile with the first pass reading the view (FROMG) and/or the
// last pass writing the view (TOG) through io; otherwise those passes run in
// shared memory like the middle ones.  The schedule must have at least one pass.
template <typename T, int EMAX, bool FROMG, bool TOG, int FX = 0>
__device__ __forceinline__ void tile_passes(typename cplx_t<T>::t *s, int ld, int nt, unsigned long long packed,
                                            const typename cplx_t<T>::t *__restrict__ twg,
                                            const uint4 *__restrict__ pc, const TileIO<T> &io) {
    typedef typename cplx_t<T>::t C;
    int fi = -1, li = 0, np = 0;
    for (int i = 0; i < kRadices; i++) {
        const int c = pass_count(packed, i);
        if (c) {
            if (fi < 0) fi = i;
            li = i;
            np += c;
        }
    }
    int Ns = 1, p = 0;
    const C *tp = twg;
    unsigned long long mid = packed;
    if (FROMG) {
        const uint4 pc0 = __ldg(&pc[0]);
        if (TOG && np == 1) {
#define JV_ONE(R) pass_first<T, R, EMAX, true, FX>(s, ld, nt, pc0, io)
            JV_RADIX_SWITCH(fi, JV_ONE)
#undef JV_ONE
            return;
        }
        int Rf = 2;
#define JV_FIRST(R) (pass_first<T, R, EMAX, false, FX>(s, ld, nt, pc0, io), Rf = R)
        JV_RADIX_SWITCH(fi, JV_FIRST)
#undef JV_FIRST
        Ns = Rf;
        p = 1;
        tp += Rf;
        mid -= 1ull << (4 * fi);
        np--;
    }
    if (TOG && np > 0) mid -= 1ull << (4 * li);
    smem_passes_from<T, EMAX>(s, ld, nt, mid, tp, pc, Ns, p);
    if (TOG && np > 0) {
        const uint4 pcl = __ldg(&pc[p]);
#define JV_LAST(R) pass_last<T, R, EMAX, FX>(s, ld, nt, Ns, tp, pcl, io)
        JV_RADIX_SWITCH(li, JV_LAST)
#undef JV_LAST
    }
}

template <typename T, int EMAX, int FX = 0>
__device__ __forceinline__ void c2c_tile(typename cplx_t<T>::t *s, int ld, int nt, unsigned long long packed,
                                         const typename cplx_t<T>::t *__restrict__ twg,
                                         const uint4 *__restrict__ pc, const TileIO<T> &io) {
    tile_passes<T, EMAX, true, true, FX>(s, ld, nt, packed, twg, pc, io);
}

// A c2c tile whose input arrived in shared memory as n*dp + t (TMA boxes of
// adjacent transforms): the first pass reads that order, the last pass
// writes the view.  The schedule must have at least two passes.
template <typename T, int EMAX, int FX = 0>
__device__ __forceinline__ void staged_tile(typename cplx_t<T>::t *s, int ld, int nt, int dp, unsigned long long packed,
                                            const typename cplx_t<T>::t *__restrict__ twg,
                                            const uint4 *__restrict__ pc, const TileIO<T> &io) {
    typedef typename cplx_t<T>::t C;
    int fi = -1, li = 0;
    for (int i = 0; i < kRadices; i++)
        if (pass_count(packed, i)) {
            if (fi < 0) fi = i;
            li = i;
        }
    const uint4 pc0 = __ldg(&pc[0]);
    int Rf = 2;
#define JV_STAGED_FIRST(R) (smem_pass<T, R, EMAX, 2>(s, ld, nt, 1, twg, pc0, dp), Rf = R)
    JV_RADIX_SWITCH(fi, JV_STAGED_FIRST)
#undef JV_STAGED_FIRST
    int Ns = Rf, p = 1;
    const C *tp = twg + Rf;
    const unsigned long long mid = packed - (1ull << (4 * fi)) - (1ull << (4 * li));
    smem_passes_from<T, EMAX>(s, ld, nt, mid, tp, pc, Ns, p);
    const uint4 pcl = __ldg(&pc[p]);
#define JV_LAST(R) pass_last<T, R, EMAX, FX>(s, ld, nt, Ns, tp, pcl, io)
    JV_RADIX_SWITCH(li, JV_LAST)
#undef JV_LAST
}

// smem_passes starting from pass p with Ns and the table pointer tp (updated)
template <typename T, int EMAX>
__device__ __forceinline__ void smem_passes_from(typename cplx_t<T>::t *s, int ld, int nt, unsigned long long packed,
                                                 const typename cplx_t<T>::t *__restrict__ &tp,
                                                 const uint4 *__restrict__ pc, int &Ns, int &p) {
#define JV_PASS_LOOP(I, R)                                                  \
    for (int q = pass_count(packed, I); q > 0; q--, p++) {                  \
        smem_pass<T, R, EMAX>(s, ld, nt, Ns, tp, __ldg(&pc[p]));            \
        tp += R * Ns;                                                       \
        Ns *= R;                                                            \
    }
    JV_PASS_LOOP(0, 16)
    JV_PASS_LOOP(1, 15)
    JV_PASS_LOOP(2, 14)
    JV_PASS_LOOP(3, 12)
    JV_PASS_LOOP(4, 10)
    JV_PASS_LOOP(5, 9)
    JV_PASS_LOOP(6, 8)
    JV_PASS_LOOP(7, 7)
    JV_PASS_LOOP(8, 6)
    JV_PASS_LOOP(9, 5)
    JV_PASS_LOOP(10, 4)
    JV_PASS_LOOP(11, 3)
    JV_PASS_LOOP(12, 2)
#undef JV_PASS_LOOP
}

// Walker over element (t, n) of a tile (t < nt transforms, n < L elements) of
// a view with vector stride vs and element stride es, from global index g0
// (transform v0, element 0).  vf: consecutive threads take consecutive
// transforms (a = n, b = t), else consecutive elements (a = t, b = n).
// exact: the launch-time constants c describe this tile (always for row
// tiles; for column tiles unless this is a shorter last tile).
__device__ __forceinline__ void walk_tile(Walk &w, bool vf, int nt, int L, long vs, long es, long g0,
                                          const WalkConst c, bool exact) {
    if (exact) {
        if (vf) w.init_c(c, es, vs, g0);
        else w.init_c(c, vs, es, g0);
    } else if (vf) {
        w.init(threadIdx.x, blockDim.x, nt, es, vs, g0);
    } else {
        w.init(threadIdx.x, blockDim.x, L, vs, es, g0);
    }
}

// Copies tot tile elements from global to shared memory (row pitch ld, padded
// index) with LB loads in flight per thread: LB addresses are walked and their
// loads issued before any of the values is stored.  get(g) reads the element
// at global index g; conj negates the imaginary parts.
template <int LB, typename C, typename Get>
__device__ __forceinline__ void tile_load(Walk &w, bool vf, int tot, C *s, int ld, bool conj, Get get) {
    const int tid = threadIdx.x, nthr = blockDim.x;
    for (int i0 = tid; i0 < tot; i0 += LB * nthr) {
        C c[LB];
        int o[LB];
#pragma unroll
        for (int u = 0; u < LB; u++) {
            const int t = vf ? w.b : w.a, n = vf ? w.a : w.b;
            o[u] = t * ld + spad(n);
            if (i0 + u * nthr < tot) c[u] = get(w.g);
            w.next();
        }
#pragma unroll
        for (int u = 0; u < LB; u++) {
            if (i0 + u * nthr < tot) {
                C v = c[u];
                if (conj) v.y = -v.y;
                s[o[u]] = v;
            }
        }
    }
}

// Instances of the shared-memory kernel beyond the three transform kinds:
// the k-omega pipeline's tapered R2C rows and power-accumulating c2c columns.
constexpr int KX_R2C_TAPER = 3, KX_C2C_POWER = 4, KX_C2C_SPLIT = 5;

template <typename T, int KIND0, int EMAX, int MAXT>
__global__ void __launch_bounds__(MAXT) k_smem(const __grid_constant__ SmemArgs<T> a) {
    typedef typename cplx_t<T>::t C;
    constexpr int KIND =
        KIND0 == KX_R2C_TAPER ? K_R2C : (KIND0 == KX_C2C_POWER || KIND0 == KX_C2C_SPLIT) ? K_C2C : KIND0;
    constexpr int FX = KIND0 == KX_R2C_TAPER   ? FX_TAPER
                       : KIND0 == KX_C2C_POWER ? FX_POWER
                       : KIND0 == KX_C2C_SPLIT ? FX_SPLIT
                                               : 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    C *s = reinterpret_cast<C *>(smem_raw);
    const int N = a.N, ld = a.ld;
    // register copies: member calls on kernel-parameter structs would force local copies
    const CAcc<T> cin = a.cin;
    const CSto<T> cout = a.cout;
    const RAcc<T> rin = a.rin;
    const RSto<T> rout = a.rout;
    const C *__restrict__ thalf = a.thalf;
    const int tid = threadIdx.x, nthr = blockDim.x;
    const long ngroups = (a.nvec + a.vpb - 1) / a.vpb;
    {
        // one CTA per group of transforms (a grid-stride loop around the
        // barrier-separated passes makes ptxas spill the codelet registers)
        const long g = blockIdx.x;
        if (g >= ngroups) return;
        const long v0 = g * a.vpb;
        const int nt = (int)min((long)a.vpb, a.nvec - v0);
        constexpr bool SPLIT = (FX & FX_SPLIT) != 0;
        if (KIND == K_C2C && a.passes != 0 &&
            (SPLIT ? (cin.cst == 1 && cout.cst == 1) : (cin.vec && cout.vec))) {
            // c2c on interleaved views: first pass from the view, last pass to the view
            TileIO<T> io;
            io.smask_in = a.conj_in ? 0x80000000u : 0u;
            io.smask_out = a.conj_out ? 0x80000000u : 0u;
            io.has_scale = a.has_scale != 0;
            io.scale = a.has_scale ? a.scale : (T)1;
            io.mnt = (nt == a.vpb) ? a.mvpb : magic_of((unsigned)nt);
            io.tw_lo = a.tw_lo;
            io.tw_hi = a.tw_hi;
            io.tw_mask = a.tw_mask;
            io.tw_sh = a.tw_sh;
            const long by = blockIdx.y;
            io.tw_t0 = (unsigned)(v0 * a.tw_ts + (a.y0 + by) * a.tw_ys);
            io.tw_ts = a.tw_ts;
            if constexpr ((FX & FX_POWER) != 0) {
                io.gram = a.gram + v0 * a.g_vs;
                io.g_es = a.g_es;
                io.g_vs = a.g_vs;
                io.g_scale = a.g_scale;
            }
            if (a.tma) {
                // column tile: TMA boxes of the vpb adjacent transforms land as n*vpb + t
                __shared__ __align__(8) uint64_t tbar;
                if (tid == 0) tc::mbar_init(&tbar, 1);
                __syncthreads();
                if (tid == 0) {
                    tc::mbar_expect_tx(&tbar, a.tma_bytes);
                    for (int i = 0; i < a.tma_boxes; i++)
                        tc::tma_load_2d(s + (size_t)i * a.tma_rows * a.vpb, &a.tmap, (int)(2 * v0),
                                        i * a.tma_rows, &tbar);
                }
                bool got = __syncthreads_and(tc::mbar_wait(&tbar, 0, 1u << 24));
                if (got && a.tma_expire) got = __syncthreads_and(tc::mbar_wait(&tbar, 1, 1u << 12));
                if (!got) {
                    if (tid == 0) atomicExch(a.status, 1);
                    return;
                }
                io.in = nullptr;
                io.in_es = io.in_vs = 0;
                io.out = reinterpret_cast<C *>(cout.re) + (cout.off + v0 * cout.vs + by * a.bvs_out);
                io.out_es = cout.es;
                io.out_vs = cout.vs;
                io.vf = true;
                io.vf_out = a.st_rows == 0;
                // the conjugation of the inverse is folded into the first pass's
                // input: flip the imaginary parts in place
                if (a.conj_in)
                    for (int i = tid; i < a.tma_boxes * a.tma_rows * a.vpb; i += nthr) s[i].y = -s[i].y;
                if (a.conj_in) __syncthreads();
                staged_tile<T, EMAX, FX>(s, ld, nt, a.vpb, a.passes, a.twg, a.pc, io);
                return;
            }
            if constexpr (SPLIT) {
                const long ei = cin.off + v0 * cin.vs + by * a.bvs_in, eo = cout.off + v0 * cout.vs + by * a.bvs_out;
                io.in_re = cin.re + ei;
                io.in_im = cin.im + ei;
                io.out_re = cout.re + eo;
                io.out_im = cout.im + eo;
                io.in = nullptr;
                io.out = nullptr;
            } else {
                io.in = reinterpret_cast<const C *>(cin.re) + (cin.off + v0 * cin.vs + by * a.bvs_in);
                io.out = reinterpret_cast<C *>(cout.re) + (cout.off + v0 * cout.vs + by * a.bvs_out);
            }
            io.in_es = cin.es;
            io.in_vs = cin.vs;
            io.out_es = cout.es;
            io.out_vs = cout.vs;
            io.vf = a.vec_fast != 0 && a.ld_rows == 0;
            io.vf_out = a.vec_fast != 0 && a.st_rows == 0;
            c2c_tile<T, EMAX, FX>(s, ld, nt, a.passes, a.twg, a.pc, io);
            return;
        }
        // ---------------- load phase
        const bool vf = a.vec_fast != 0;
        const bool exact = !vf || nt == a.vpb;
        const WalkConst win = a.win, wout = a.wout;
        constexpr int LB = (sizeof(T) == 4 && EMAX <= 8) ? 8 : 4;  // loads in flight per thread
        // real rows of unit stride, even offset and pitch: x_{2n}, x_{2n+1} are
        // one interleaved complex element, so the R2C first pass reads them
        // from the view and the C2R last pass writes them to the view
        const bool rp = (KIND != K_C2C) && a.real_pairs && a.passes != 0;
        Walk w;
        if (KIND == K_R2C && rp) {
            TileIO<T> io;
            io.in = reinterpret_cast<const C *>(rin.a + (rin.off + v0 * rin.vs));
            io.out = nullptr;
            io.in_es = 1;
            io.in_vs = rin.vs / 2;
            io.out_es = io.out_vs = 0;
            io.smask_in = io.smask_out = 0u;
            io.has_scale = false;
            io.scale = (T)1;
            io.vf = io.vf_out = false;
            io.mnt = 0;
            io.tw_lo = io.tw_hi = nullptr;
            if constexpr ((FX & FX_TAPER) != 0) {
                io.tp_n = a.tp_n;
                io.tp_n_st = a.tp_n_st;
                io.tp_t = a.tp_t + v0 * a.tp_t_st;
                io.tp_t_st = a.tp_t_st;
                io.wb = a.tp_back ? const_cast<C *>(io.in) : nullptr;
            }
            tile_passes<T, EMAX, true, false, FX>(s, ld, nt, a.passes, a.twg, a.pc, io);
        } else {
        if (KIND == K_C2C) {
            walk_tile(w, vf, nt, N, cin.vs, cin.es, cin.off + v0 * cin.vs, win, exact);
            tile_load<LB>(w, vf, nt * N, s, ld, a.inv != 0, [&](long g) { return cin.at(g); });
        } else if (KIND == K_R2C) {
            // z_n = x_{2n} + i x_{2n+1}  (c_VSIP_src/VI_rcfftmop_f_def.h:53-75)
            walk_tile(w, vf, nt, N, rin.vs, 2 * rin.es, rin.off + v0 * rin.vs, win, exact);
            tile_load<LB>(w, vf, nt * N, s, ld, false,
                          [&](long g) { return mk<C>(rin.a[rin.rst * g], rin.a[rin.rst * (g + rin.es)]); });
        } else {
            // C2R: raw Z_k, k <= N, then the inverse split (VI_crfftmop_f_def.h:58-110)
            walk_tile(w, vf, nt, N + 1, cin.vs, cin.es, cin.off + v0 * cin.vs, win, exact);
            tile_load<LB>(w, vf, nt * (N + 1), s, ld, false, [&](long g) { return cin.at(g); });
            __syncthreads();
            const int half = N / 2 + 1;   // pairs (k, N-k), k = 0..N/2
            const int totp = nt * half;
            const unsigned mh = magic_of((unsigned)half);
            for (int i = tid; i < totp; i += nthr) {
                int t = mdiv(i, mh), k = i - t * half;
                C *row = s + t * ld;
                C f = row[spad(k)], b = row[spad(N - k)];
                C h = thalf[k];
                // Y_k = f + b + w.i (b - f) ... with f = Z_k, b = Z_{N-k}, w = exp(+i pi k/N)
                C yk = mk<C>(f.x + b.x + h.y * (b.x - f.x) - h.x * (f.y + b.y),
                             f.y - b.y - h.y * (f.y + b.y) + h.x * (f.x - b.x));
                C yn;
                bool pair = (k != 0) && (N - k != k);
                if (pair) {
                    C w2 = thalf[N - k];
                    yn = mk<C>(b.x + f.x + w2.y * (f.x - b.x) - w2.x * (b.y + f.y),
                               b.y - f.y - w2.y * (b.y + f.y) + w2.x * (b.x - f.x));
                }
                // the inverse transform runs as a forward one on conjugated data
                row[spad(k)] = mk<C>(yk.x, -yk.y);
                if (pair) row[spad(N - k)] = mk<C>(yn.x, -yn.y);
            }
        }
        __syncthreads();
        if (KIND == K_C2R && rp) {
            // x_{2n} = Re y_n, x_{2n+1} = Im y_n (VI_crfftmop_f_def.h:121-124)
            // written by the last pass: y conjugated back, scaled
            TileIO<T> io;
            io.in = nullptr;
            io.out = reinterpret_cast<C *>(rout.a + (rout.off + v0 * rout.vs));
            io.in_es = io.in_vs = 0;
            io.out_es = 1;
            io.out_vs = rout.vs / 2;
            io.smask_in = 0u;
            io.smask_out = 0x80000000u;
            io.has_scale = a.has_scale != 0;
            io.scale = a.has_scale ? a.scale : (T)1;
            io.vf = io.vf_out = false;
            io.mnt = 0;
            io.tw_lo = io.tw_hi = nullptr;
            tile_passes<T, EMAX, false, true>(s, ld, nt, a.passes, a.twg, a.pc, io);
            return;
        }
        // ---------------- radix passes
        smem_passes<T, EMAX>(s, ld, nt, a.passes, a.twg, a.pc);
        }
        // ---------------- store phase
        if (KIND == K_C2C) {
            const int tot = nt * N;
            walk_tile(w, vf, nt, N, cout.vs, cout.es, cout.off + v0 * cout.vs, wout, exact);
            for (int i = tid; i < tot; i += nthr, w.next()) {
                const int t = vf ? w.b : w.a, n = vf ? w.a : w.b;
                C c = s[t * ld + spad(n)];
                if (a.inv) c.y = -c.y;
                if (a.has_scale) c = cscale(c, a.scale);
                cout.put(w.g, c);
            }
        } else if (KIND == K_R2C) {
            // Hermitian split (VI_rcfftmop_f_def.h:79-118): X_k from Z_k and Z_{N-k} (Z_N = Z_0)
            const int tot = nt * (N + 1);
            walk_tile(w, vf, nt, N + 1, cout.vs, cout.es, cout.off + v0 * cout.vs, wout, exact);
            for (int i = tid; i < tot; i += nthr, w.next()) {
                const int t = vf ? w.b : w.a, k = vf ? w.a : w.b;
                const C *row = s + t * ld;
                C f = row[spad(k == N ? 0 : k)];
                C b = row[spad(k == 0 ? 0 : N - k)];
                if (a.has_scale) {
                    f = cscale(f, a.scale);
                    b = cscale(b, a.scale);
                }
                C h = thalf[k];
                C x = mk<C>((T)0.5 * (b.x + f.x + h.x * (b.y + f.y) + h.y * (f.x - b.x)),
                            (T)0.5 * (f.y - b.y + h.x * (b.x - f.x) + h.y * (b.y + f.y)));
                cout.put(w.g, x);
            }
        } else {
            // x_{2n} = Re y_n, x_{2n+1} = Im y_n (VI_crfftmop_f_def.h:121-124)
            const int tot = nt * N;
            walk_tile(w, vf, nt, N, rout.vs, 2 * rout.es, rout.off + v0 * rout.vs, wout, exact);
            for (int i = tid; i < tot; i += nthr, w.next()) {
                const int t = vf ? w.b : w.a, n = vf ? w.a : w.b;
                C c = s[t * ld + spad(n)];
                T re = c.x, im = -c.y;
                if (a.has_scale) {
                    re *= a.scale;
                    im *= a.scale;
                }
                rout.a[rout.rst * w.g] = re;
                rout.a[rout.rst * (w.g + rout.es)] = im;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- global pass kernel
// One radix-R pass of every transform: src -> dst, both given as views in
// transform order.  R is a codelet radix or any odd prime (O(R^2) direct sum).
template <typename T> struct GPassArgs {
    typedef typename cplx_t<T>::t C;
    int N, R, Ns;
    long nvec;
    int conj_in, conj_out;  // conjugate on read / write
    int has_scale;
    T scale;
    int src_real;           // src is a real view read as z_n = x_2n + i x_2n+1
    CAcc<T> src;
    RAcc<T> rsrc;
    CSto<T> dst;
    const C *tw;
};

template <typename T, int R>
__device__ __forceinline__ void gpass_body(const GPassArgs<T> &a, long v, int j) {
    typedef typename cplx_t<T>::t C;
    const int NR = a.N / R;
    C x[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        C c;
        if (a.src_real) c = mk<C>(a.rsrc.load(v, 2 * (j + r * NR)), a.rsrc.load(v, 2 * (j + r * NR) + 1));
        else c = a.src.load(v, j + r * NR);
        if (a.conj_in) c.y = -c.y;
        x[r] = c;
    }
    int m = j % a.Ns;
    if (m) {
        long st = (long)m * (a.N / (a.Ns * R));
#pragma unroll
        for (int r = 1; r < R; r++) x[r] = cmul(x[r], __ldg(&a.tw[r * st]));
    }
    Dft<C, R>::run(x);
    long base = (long)(j - m) * R + m;
#pragma unroll
    for (int r = 0; r < R; r++) {
        C c = x[r];
        if (a.conj_out) c.y = -c.y;
        if (a.has_scale) c = cscale(c, a.scale);
        a.dst.store(v, base + (long)r * a.Ns, c);
    }
}

// Radices with a codelet; any other radix is an odd prime, taken by the
// odd-prime codelet up to 23 and as a direct sum above.
__host__ __device__ __forceinline__ bool gpass_codelet(int R) {
    return R == 2 || R == 3 || R == 4 || R == 5 || R == 6 || R == 7 || R == 8 || R == 9 || R == 10 || R == 12 ||
           R == 14 || R == 15 || R == 16;
}
__host__ __device__ __forceinline__ bool gpass_prime(int R) {
    return R == 11 || R == 13 || R == 17 || R == 19 || R == 23;
}

// Output k of butterfly j of a prime-radix pass as the direct sum over its R
// inputs (the O(R^2) DFT of c_VSIP_src/VI_fftm_building_blocks_f.h:95-155,
// VI_dftm_f, with the inter-pass twiddle folded into the load).  One thread
// per output keeps the work of a thread at R complex multiply-adds, so a
// transform of prime length spreads over N threads.
template <typename T>
__device__ __forceinline__ void gpass_generic(const GPassArgs<T> &a, long v, int j, int k) {
    typedef typename cplx_t<T>::t C;
    const int R = a.R, NR = a.N / R;
    const int m = j % a.Ns;
    const long st = (long)m * (a.N / (a.Ns * R));
    const long base = (long)(j - m) * R + m;
    const long rstep = a.N / R;  // table index step of exp(-2 pi i/R)
    C acc = mk<C>((T)0, (T)0);
    int e = 0;                   // (n * k) mod R
    for (int n = 0; n < R; n++) {
        C c;
        if (a.src_real) c = mk<C>(a.rsrc.load(v, 2 * (j + n * NR)), a.rsrc.load(v, 2 * (j + n * NR) + 1));
        else c = a.src.load(v, j + n * NR);
        if (a.conj_in) c.y = -c.y;
        if (m && n) c = cmul(c, __ldg(&a.tw[n * st]));
        C w = __ldg(&a.tw[(long)e * rstep]);
        acc = cadd(acc, cmul(c, w));
        e += k;
        if (e >= R) e -= R;
    }
    if (a.conj_out) acc.y = -acc.y;
    if (a.has_scale) acc = cscale(acc, a.scale);
    a.dst.store(v, base + (long)k * a.Ns, acc);
}

// Work items of one pass: a butterfly (j) for codelet radices, an output
// (j, k) of a butterfly for direct-sum radices.
__host__ __device__ __forceinline__ long gpass_items(long nvec, int N, int R) {
    return (gpass_codelet(R) || gpass_prime(R)) ? nvec * (N / R) : nvec * (long)N;
}

// A pass of a radix R with a codelet (prime R <= 23 included): one thread
// per butterfly, the R inputs loaded once.  One kernel instance per radix, so
// each runs with its own codelet's registers (radix 8: 44 per thread, five
// 256-thread CTAs per SM, against 61 and four for a kernel switching over
// every radix: 1.5x on 4096 x 5632 = 8^3 x 11).
template <typename T, int R>
__global__ void __launch_bounds__(256) k_gpass_r(const GPassArgs<T> pa) {
    const GPassArgs<T> a = pa;
    const long NR = a.N / R;
    const long total = a.nvec * NR;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const long v = i / NR;
        gpass_body<T, R>(a, v, (int)(i - v * NR));
    }
}

// Shared-memory pitch (elements) of a thread's R outputs in the first pass's
// staging: odd, so a half-warp's 64-bit stores hit distinct banks.
template <int R> __host__ __device__ constexpr int gpass_stage_pitch() { return R | 1; }

// The first pass (Ns = 1) of a multi-pass transform: butterfly j writes its R
// outputs to j*R .. j*R + R - 1, so a CTA's 256 consecutive butterflies
// (i = v*N/R + j over the transforms) fill the contiguous outputs
// [i0*R, (i0 + 256)*R) of the flattened (v, n) output space.  They go through
// shared memory (with each slot's transform and butterfly, so the stores need
// no division) and leave as 256-element coalesced runs instead of R elements
// 8*R bytes apart per store instruction.  Every thread of the CTA
// runs the same loop trips (the barriers), with its own butterfly when it has one.
template <typename T, int R>
__global__ void __launch_bounds__(256) k_gpass_r1(const GPassArgs<T> pa) {
    typedef typename cplx_t<T>::t C;
    extern __shared__ __align__(16) unsigned char gsm_raw[];
    C *stg = reinterpret_cast<C *>(gsm_raw);
    __shared__ long bv[256];  // transform and butterfly of each staged slot
    __shared__ int bj[256];
    constexpr int P = gpass_stage_pitch<R>();
    const GPassArgs<T> a = pa;
    const long NR = a.N / R;
    const long total = a.nvec * NR;
    const int t = threadIdx.x;
    for (long i0 = (long)blockIdx.x * 256; i0 < total; i0 += (long)gridDim.x * 256) {
        const long i = i0 + t;
        if (i < total) {
            const long v = i / NR;
            const int j = (int)(i - v * NR);
            bv[t] = v;
            bj[t] = j;
            C x[R];
#pragma unroll
            for (int r = 0; r < R; r++) {
                C c;
                if (a.src_real) c = mk<C>(a.rsrc.load(v, 2 * (j + r * NR)), a.rsrc.load(v, 2 * (j + r * NR) + 1));
                else c = a.src.load(v, j + r * NR);
                if (a.conj_in) c.y = -c.y;
                x[r] = c;
            }
            Dft<C, R>::run(x);
#pragma unroll
            for (int r = 0; r < R; r++) {
                C c = x[r];
                if (a.conj_out) c.y = -c.y;
                if (a.has_scale) c = cscale(c, a.scale);
                stg[t * P + r] = c;
            }
        }
        __syncthreads();
        const int cnt = (int)(total - i0 < 256 ? total - i0 : 256) * R;  // outputs of this trip
        for (int e = t; e < cnt; e += 256) {
            // output r of staged butterfly q: element j*R + r of its transform
            const int q = e / R, r = e - q * R;
            a.dst.store(bv[q], (long)bj[q] * R + r, stg[q * P + r]);
        }
        __syncthreads();
    }
}

// A pass of a prime radix above 23 as direct sums, one thread per output.
template <typename T>
__global__ void __launch_bounds__(256) k_gpass(const GPassArgs<T> pa) {
    const GPassArgs<T> a = pa;
    const long NR = a.N / a.R;
    // consecutive threads take consecutive butterflies j of one output k,
    // so their loads of input n are adjacent
    const long total = a.nvec * (long)a.N;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        long v = i / a.N;
        long rem = i - v * a.N;
        int k = (int)(rem / NR);
        int j = (int)(rem - (long)k * NR);
        gpass_generic<T>(a, v, j, k);
    }
}

// R2C Hermitian split / C2R un-split on dense scratch for the global path.
template <typename T> struct SplitArgs {
    typedef typename cplx_t<T>::t C;
    int N;          // half length MN
    long nvec;
    int has_scale;
    T scale;
    const C *zsrc;  // R2C: transformed Z (dense [nvec][N]); C2R: unused
    CAcc<T> zin;    // C2R: input spectrum view (N+1 per transform)
    CSto<T> xout;   // R2C: output spectrum view (N+1 per transform)
    C *ydst;        // C2R: dense [nvec][N] conjugated Y for the forward passes
    const C *thalf;
};

template <typename T>
__global__ void k_r2c_split(const SplitArgs<T> a) {
    typedef typename cplx_t<T>::t C;
    const long tot = a.nvec * (a.N + 1);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
        long v = i / (a.N + 1);
        int k = (int)(i - v * (a.N + 1));
        const C *row = a.zsrc + v * a.N;
        C f = row[k == a.N ? 0 : k];
        C b = row[k == 0 ? 0 : a.N - k];
        if (a.has_scale) {
            f = cscale(f, a.scale);
            b = cscale(b, a.scale);
        }
        C w = a.thalf[k];
        C x = mk<C>((T)0.5 * (b.x + f.x + w.x * (b.y + f.y) + w.y * (f.x - b.x)),
                    (T)0.5 * (f.y - b.y + w.x * (b.x - f.x) + w.y * (b.y + f.y)));
        a.xout.store(v, k, x);
    }
}

template <typename T>
__global__ void k_c2r_unsplit(const SplitArgs<T> a) {
    typedef typename cplx_t<T>::t C;
    const long tot = a.nvec * a.N;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
        long v = i / a.N;
        int k = (int)(i - v * a.N);
        C f = a.zin.load(v, k), b = a.zin.load(v, a.N - k);
        C w = a.thalf[k];
        C y = mk<C>(f.x + b.x + w.y * (b.x - f.x) - w.x * (f.y + b.y),
                    f.y - b.y - w.y * (f.y + b.y) + w.x * (f.x - b.x));
        a.ydst[v * a.N + k] = mk<C>(y.x, -y.y);
    }
}

// R2C Hermitian split in place on an interleaved output view holding Z_k,
// k < N (the two steps of a long transform wrote it there): the thread of pair
// k (0 <= k <= N/2) reads Z_k and Z_{N-k} (Z_N = Z_0) and writes X_k and
// X_{N-k} (X_N for k = 0), so no thread reads what another writes
// (c_VSIP_src/VI_rcfftmop_f_def.h:79-118).
template <typename T> struct PairSplitArgs {
    typedef typename cplx_t<T>::t C;
    C *z;           // element (v, k) at z[v*vs + k*es]
    long es, vs;
    int N;
    long nvec;
    int has_scale;
    T scale;
    const C *thalf;
};

template <typename T>
__global__ void k_r2c_split_pairs(const PairSplitArgs<T> a) {
    typedef typename cplx_t<T>::t C;
    const int H = a.N / 2 + 1;
    const long tot = a.nvec * H;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
        const long v = i / H;
        const int k = (int)(i - v * H);
        C *row = a.z + v * a.vs;
        const int nk = (k == 0) ? a.N : a.N - k;  // output index of the pair's second element
        C zk = row[(long)k * a.es];
        C zn = row[(long)(k == 0 ? 0 : a.N - k) * a.es];
        if (a.has_scale) {
            zk = cscale(zk, a.scale);
            zn = cscale(zn, a.scale);
        }
        const C w = a.thalf[k], w2 = a.thalf[nk];
        // X_k from f = Z_k, b = Z_{N-k}; X_{N-k} from f = Z_{N-k}, b = Z_k
        const C xk = mk<C>((T)0.5 * (zn.x + zk.x + w.x * (zn.y + zk.y) + w.y * (zk.x - zn.x)),
                           (T)0.5 * (zk.y - zn.y + w.x * (zn.x - zk.x) + w.y * (zn.y + zk.y)));
        const C xn = mk<C>((T)0.5 * (zk.x + zn.x + w2.x * (zk.y + zn.y) + w2.y * (zn.x - zk.x)),
                           (T)0.5 * (zn.y - zk.y + w2.x * (zk.x - zn.x) + w2.y * (zk.y + zn.y)));
        row[(long)k * a.es] = xk;
        if (nk != k) row[(long)nk * a.es] = xn;
    }
}

// C2R final store from dense conjugated y: x_2n = Re, x_2n+1 = -Im (conj back), scaled.
template <typename T> struct UnpackArgs {
    typedef typename cplx_t<T>::t C;
    int N;
    long nvec;
    int has_scale;
    T scale;
    const C *y;
    RSto<T> xout;
};

template <typename T>
__global__ void k_c2r_unpack(const UnpackArgs<T> a) {
    typedef typename cplx_t<T>::t C;
    const long tot = a.nvec * a.N;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < tot; i += (long)gridDim.x * blockDim.x) {
        long v = i / a.N;
        int n = (int)(i - v * a.N);
        C c = a.y[i];
        T re = c.x, im = -c.y;
        if (a.has_scale) {
            re *= a.scale;
            im *= a.scale;
        }
        a.xout.store(v, 2 * n, re);
        a.xout.store(v, 2 * n + 1, im);
    }
}

}  // namespace jv
