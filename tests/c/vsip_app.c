/* vsip_app.c -- a C89 VSIPL application of the fftm and single-FFT calls,
 * built against include/vsip_fftm_gb300.h and linked with the GPU library
 * only (tests/test_c_app.py).  It binds user data, admits the blocks, runs
 * vsip_ccfftmop_f (VSIP_ROW), vsip_ccfftmip_f (VSIP_COL, inverse, scaled),
 * vsip_rcfftmop_f and vsip_ccfftop_d, releases the blocks and compares each
 * result with a direct DFT in double precision.  Exit status 0 when every
 * relative error is within the acceptance tolerance. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "vsip_fftm_gb300.h"

#define PI 3.14159265358979323846

/* y_k = scale * sum_n x_n exp(dir 2 pi i n k / N), interleaved, strides in complex elements */
static void dft(const double *x, long xs, double *y, long ys, long N, int dir, double scale) {
    long k, n;
    for (k = 0; k < N; k++) {
        double re = 0.0, im = 0.0;
        for (n = 0; n < N; n++) {
            double a = dir * 2.0 * PI * (double)((n * k) % N) / (double)N;
            double c = cos(a), s = sin(a);
            re += x[2 * n * xs] * c - x[2 * n * xs + 1] * s;
            im += x[2 * n * xs] * s + x[2 * n * xs + 1] * c;
        }
        y[2 * k * ys] = scale * re;
        y[2 * k * ys + 1] = scale * im;
    }
}

static double relerr_f(const float *got, const double *ref, long n) {
    double num = 0.0, den = 0.0;
    long i;
    for (i = 0; i < n; i++) {
        double d = (double)got[i] - ref[i];
        num += d * d;
        den += ref[i] * ref[i];
    }
    return sqrt(num / den);
}

static double lcg(unsigned long *s) {
    *s = *s * 6364136223846793005UL + 1442695040888963407UL;
    return (double)((*s >> 11) & ((1UL << 53) - 1)) / 9007199254740992.0 * 2.0 - 1.0;
}

int main(void) {
    const long M = 6, N = 96;
    unsigned long seed = 12345;
    long i, r, c;
    int fails = 0;
    float *x = (float *)malloc(sizeof(float) * 2 * M * N), *y = (float *)malloc(sizeof(float) * 2 * M * N);
    double *xd = (double *)malloc(sizeof(double) * 2 * M * N), *ref = (double *)malloc(sizeof(double) * 2 * M * N);
    vsip_cblock_f *bx, *by;
    vsip_cmview_f *vx, *vy;
    vsip_fftm_f *rows, *cols;
    double e;

    if (vsip_init(NULL) != 0) {
        printf("vsip_init failed\n");
        return 2;
    }
    for (i = 0; i < 2 * M * N; i++) {
        xd[i] = lcg(&seed);
        x[i] = (float)xd[i];
        xd[i] = (double)x[i];
    }
    bx = vsip_cblockbind_f(x, NULL, (vsip_length)(M * N), VSIP_MEM_NONE);
    by = vsip_cblockbind_f(y, NULL, (vsip_length)(M * N), VSIP_MEM_NONE);
    vsip_cblockadmit_f(bx, 1);
    vsip_cblockadmit_f(by, 0);
    vx = vsip_cmbind_f(bx, 0, (vsip_stride)N, (vsip_length)M, 1, (vsip_length)N);
    vy = vsip_cmbind_f(by, 0, (vsip_stride)N, (vsip_length)M, 1, (vsip_length)N);

    /* rows, forward */
    rows = vsip_ccfftmop_create_f((vsip_length)M, (vsip_length)N, 1.0f, VSIP_FFT_FWD, VSIP_ROW, 0, VSIP_ALG_TIME);
    if (!rows) {
        printf("create failed: %s\n", jvsip_gpu_last_error_string());
        return 2;
    }
    vsip_ccfftmop_f(rows, vx, vy);
    vsip_cblockrelease_f(by, 1, NULL, NULL);
    for (r = 0; r < M; r++) dft(xd + 2 * r * N, 1, ref + 2 * r * N, 1, N, -1, 1.0);
    e = relerr_f(y, ref, 2 * M * N);
    printf("ccfftmop_f rows     rel-L2 %.3e\n", e);
    fails += !(e <= 1e-6 * log((double)N) / log(2.0));

    /* columns of y in place: inverse with scale 1/M */
    vsip_cblockadmit_f(by, 1);
    cols = vsip_ccfftmip_create_f((vsip_length)M, (vsip_length)N, (vsip_scalar_f)(1.0 / M), VSIP_FFT_INV, VSIP_COL, 0,
                                  VSIP_ALG_TIME);
    vsip_ccfftmip_f(cols, vy);
    vsip_cblockrelease_f(by, 1, NULL, NULL);
    {
        double *tmp = (double *)malloc(sizeof(double) * 2 * M * N);
        for (c = 0; c < N; c++) dft(ref + 2 * c, N, tmp + 2 * c, N, M, +1, 1.0 / M);
        e = relerr_f(y, tmp, 2 * M * N);
        free(tmp);
    }
    printf("ccfftmip_f columns  rel-L2 %.3e\n", e);
    fails += !(e <= 1e-6 * 8);

    /* real rows -> half spectra */
    {
        const long Nr = 2 * N, H = N + 1;
        float *xr = (float *)malloc(sizeof(float) * M * Nr), *z = (float *)malloc(sizeof(float) * 2 * M * H);
        double *cx = (double *)malloc(sizeof(double) * 2 * Nr), *cz = (double *)malloc(sizeof(double) * 2 * Nr);
        double num = 0.0, den = 0.0;
        vsip_block_f *br = vsip_blockbind_f(xr, (vsip_length)(M * Nr), VSIP_MEM_NONE);
        vsip_cblock_f *bz = vsip_cblockbind_f(z, NULL, (vsip_length)(M * H), VSIP_MEM_NONE);
        vsip_mview_f *vr = vsip_mbind_f(br, 0, (vsip_stride)Nr, (vsip_length)M, 1, (vsip_length)Nr);
        vsip_cmview_f *vz = vsip_cmbind_f(bz, 0, (vsip_stride)H, (vsip_length)M, 1, (vsip_length)H);
        vsip_fftm_f *rc = vsip_rcfftmop_create_f((vsip_length)M, (vsip_length)Nr, 1.0f, VSIP_ROW, 0, VSIP_ALG_TIME);
        for (i = 0; i < M * Nr; i++) xr[i] = (float)lcg(&seed);
        vsip_blockadmit_f(br, 1);
        vsip_cblockadmit_f(bz, 0);
        vsip_rcfftmop_f(rc, vr, vz);
        vsip_cblockrelease_f(bz, 1, NULL, NULL);
        for (r = 0; r < M; r++) {
            long k;
            for (i = 0; i < Nr; i++) {
                cx[2 * i] = xr[r * Nr + i];
                cx[2 * i + 1] = 0.0;
            }
            dft(cx, 1, cz, 1, Nr, -1, 1.0);
            for (k = 0; k < H; k++) {
                double dr = z[2 * (r * H + k)] - cz[2 * k], di = z[2 * (r * H + k) + 1] - cz[2 * k + 1];
                num += dr * dr + di * di;
                den += cz[2 * k] * cz[2 * k] + cz[2 * k + 1] * cz[2 * k + 1];
            }
        }
        e = sqrt(num / den);
        printf("rcfftmop_f rows     rel-L2 %.3e\n", e);
        fails += !(e <= 1e-6 * 8);
        vsip_mdestroy_f(vr);
        vsip_cmdestroy_f(vz);
        vsip_blockrelease_f(br, 0);
        vsip_blockdestroy_f(br);
        vsip_cblockdestroy_f(bz);
        vsip_fftm_destroy_f(rc);
        free(xr);
        free(z);
        free(cx);
        free(cz);
    }

    /* a single FFT in double precision on a strided vector (not admitted: staged) */
    {
        const long L = 360;
        double *v = (double *)malloc(sizeof(double) * 2 * 2 * L), *w = (double *)malloc(sizeof(double) * 2 * L);
        double *cref = (double *)malloc(sizeof(double) * 2 * L);
        double num = 0.0, den = 0.0;
        vsip_cblock_d *bv = vsip_cblockbind_d(v, NULL, (vsip_length)(2 * L), VSIP_MEM_NONE);
        vsip_cblock_d *bw = vsip_cblockbind_d(w, NULL, (vsip_length)L, VSIP_MEM_NONE);
        vsip_cvview_d *cv = vsip_cvbind_d(bv, 1, 2, (vsip_length)L);
        vsip_cvview_d *cw = vsip_cvbind_d(bw, 0, 1, (vsip_length)L);
        vsip_fft_d *f = vsip_ccfftop_create_d((vsip_length)L, 0.5, VSIP_FFT_FWD, 1, VSIP_ALG_TIME);
        vsip_fft_attr_d at;
        for (i = 0; i < 4 * L; i++) v[i] = lcg(&seed);
        vsip_fft_getattr_d(f, &at);
        vsip_ccfftop_d(f, cv, cw);
        dft(v + 2, 2, cref, 1, L, -1, 0.5);
        for (i = 0; i < 2 * L; i++) {
            num += (w[i] - cref[i]) * (w[i] - cref[i]);
            den += cref[i] * cref[i];
        }
        e = sqrt(num / den);
        printf("ccfftop_d vector    rel-L2 %.3e  (attr input %lu output %lu place %d)\n", e,
               (unsigned long)at.input, (unsigned long)at.output, (int)at.place);
        fails += !(e <= 1e-14 * 9) + !(at.input == (vsip_scalar_vi)L && at.output == (vsip_scalar_vi)L);
        vsip_cvdestroy_d(cv);
        vsip_cvdestroy_d(cw);
        vsip_cblockdestroy_d(bv);
        vsip_cblockdestroy_d(bw);
        vsip_fft_destroy_d(f);
        free(v);
        free(w);
        free(cref);
    }

    vsip_cmdestroy_f(vx);
    vsip_cmdestroy_f(vy);
    vsip_cblockrelease_f(bx, 0, NULL, NULL);
    vsip_cblockdestroy_f(bx);
    vsip_cblockdestroy_f(by);
    vsip_fftm_destroy_f(rows);
    vsip_fftm_destroy_f(cols);
    if (jvsip_gpu_last_error()) {
        printf("library error: %s\n", jvsip_gpu_last_error_string());
        fails++;
    }
    vsip_finalize(NULL);
    free(x);
    free(y);
    free(xd);
    free(ref);
    printf(fails ? "FAIL\n" : "OK\n");
    return fails ? 1 : 0;
}
