/*
 * fftm_oracle.c -- CPU oracle for the VSIPL multiple-FFT calls.
 * TEST INFRASTRUCTURE ONLY (see fftm_oracle.h): the tests, the smoke check and
 * the CPU-baseline leg of the benchmark load it; the GPU library never does.
 *
 * Build (both hosts):  gcc -O2 -std=c99 -fPIC -ffp-contract=off -shared
 *                      -o oracle/liborc_fftm.so oracle/fftm_oracle.c -lm -lpthread
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include "fftm_oracle.h"

/* Factorisation of c_VSIP_src/VI_nuV.h:22-136: all 3s, then 5s, 7s, 8s, 4s,
 * 2s; each found radix is one stage with pn = count (+1 when a cofactor
 * remains, the cofactor becoming that stage's final radix pF).  A length with
 * no supported factor is one stage (p0 = 1, pF = N): a plain DFT. */
unsigned long orc_factor(unsigned long N, unsigned long *pn, unsigned long *p0, unsigned long *pF)
{
    static const unsigned long radix[6] = {3, 5, 7, 8, 4, 2};
    unsigned long n = N, k = 0;
    int r;
    if (N == 0) return 0;
    for (r = 0; r < 6; r++) {
        unsigned long q = radix[r], cnt = 0;
        while (n % q == 0) { n /= q; cnt++; }
        if (cnt) {
            p0[k] = q;
            if (n != 1) { pF[k] = n; pn[k] = cnt + 1; }
            else        { pF[k] = q; pn[k] = cnt; }
            k++;
        }
    }
    if (n != 1 && k == 0) { p0[0] = 1; pF[0] = n; pn[0] = 1; k = 1; }
    return k;
}

/* Mixed-radix digit reversal of c_VSIP_src/VI_jofk.h:21-48 (Van Loan 2.2.3). */
unsigned long orc_jofk(unsigned long k, const unsigned long *pn, const unsigned long *p0,
                       unsigned long pF, unsigned long nstage)
{
    unsigned long j = 0, m = k, q, i;
    for (q = 0; q < nstage; q++) {
        unsigned long p = p0[q];
        for (i = 1; i < pn[q]; i++) {
            unsigned long s = m / p;
            j = p * j + (m - s * p);
            m = s;
        }
    }
    {
        unsigned long s = m / pF;
        j = pF * j + (m - s * pF);
    }
    return j;
}

/* ---- seeded synthetic inputs ---- */
static unsigned long long orc_mix(unsigned long long seed, unsigned long long idx)
{
    unsigned long long z = seed * 0xD1342543DE82EF95ULL + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double orc_unit(unsigned long long seed, unsigned long long idx)
{
    return (double)(orc_mix(seed, idx) >> 11) * (1.0 / 9007199254740992.0);
}

static double orc_sample(unsigned long long seed, unsigned long i, int dist)
{
    if (dist == 0) return 2.0 * orc_unit(seed, i) - 1.0;
    {
        unsigned long long pair = (unsigned long long)(i / 2) * 2ULL;
        double u1 = orc_unit(seed, pair), u2 = orc_unit(seed, pair + 1);
        double r = sqrt(-2.0 * log(1.0 - u1));
        double t = 6.283185307179586476925286766559 * u2;
        return (i & 1) ? r * sin(t) : r * cos(t);
    }
}

void orc_fill_f(float *dst, unsigned long n, unsigned long long seed, int dist)
{
    unsigned long i;
    for (i = 0; i < n; i++) dst[i] = (float)orc_sample(seed, i, dist);
}

void orc_fill_d(double *dst, unsigned long n, unsigned long long seed, int dist)
{
    unsigned long i;
    for (i = 0; i < n; i++) dst[i] = orc_sample(seed, i, dist);
}

#define T float
#define SFX _f
#include "fftm_oracle_body.h"
#undef T
#undef SFX

#define T double
#define SFX _d
#include "fftm_oracle_body.h"
#undef T
#undef SFX
