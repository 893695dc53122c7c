/*
 * fftm_oracle.h -- CPU oracle for the VSIPL multiple-FFT calls.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the jvsip
 * reference's default (non-FFTW) fftm algorithm: the VI_nuV factorisation,
 * the recursive mixed-radix decimation-in-frequency stage driver with the
 * batch loop innermost, the separate twiddle pass, the O(L^2) DFT for
 * unsupported factors, the jofk digit-reversal gather, the scale pass and the
 * real<->complex packing.  It follows the reference's arithmetic order so that
 * its results match the reference bit for bit (checked against the reference
 * library built from source and against the reference's own fixtures).
 *
 * It is used by the tests as the checker, by __graft_entry__.smoke() as the
 * checker, and by bench.py as the timed CPU baseline.  The GPU library never
 * links, loads or calls it.
 */
#ifndef FFTM_ORACLE_H
#define FFTM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* transform kinds, as c_VSIP_src/VI_ffttype.h */
#define ORC_CCOP 0
#define ORC_CCIP 1
#define ORC_RCOP 2
#define ORC_CROP 3

/* A complex matrix view: element (i,j) has its real part at
 * re[cst*(off + i*col_stride + j*row_stride)] and its imaginary part at the
 * same index of im.  Interleaved data: im = re + 1, cst = 2.  Split: cst = 1.
 * (c_VSIP_src/vsip_cmviewattributes_f.h:47-55, vsip_cblockattributes_f.h:42-67) */
typedef struct { float  *re, *im; long cst, off, col_stride, row_stride;
                 unsigned long col_length, row_length; } orc_cmview_f;
typedef struct { double *re, *im; long cst, off, col_stride, row_stride;
                 unsigned long col_length, row_length; } orc_cmview_d;
/* A real matrix view: element (i,j) at a[rst*(off + i*col_stride + j*row_stride)]
 * (c_VSIP_src/vsip_mviewattributes_f.h:47-55, vsip_blockattributes_f.h:40-51) */
typedef struct { float  *a; long rst, off, col_stride, row_stride;
                 unsigned long col_length, row_length; } orc_mview_f;
typedef struct { double *a; long rst, off, col_stride, row_stride;
                 unsigned long col_length, row_length; } orc_mview_d;

typedef struct orc_fftm_f orc_fftm_f;
typedef struct orc_fftm_d orc_fftm_d;

/* kind: ORC_CCOP/CCIP/RCOP/CROP; dir is ignored for RCOP (forward) and CROP (inverse). */
orc_fftm_f *orc_fftm_create_f(int kind, unsigned long M, unsigned long N, float scale,
                              int dir, int major);
orc_fftm_d *orc_fftm_create_d(int kind, unsigned long M, unsigned long N, double scale,
                              int dir, int major);
void orc_fftm_destroy_f(orc_fftm_f *p);
void orc_fftm_destroy_d(orc_fftm_d *p);

void orc_ccfftmop_f(const orc_fftm_f *p, const orc_cmview_f *x, const orc_cmview_f *y);
void orc_ccfftmip_f(const orc_fftm_f *p, const orc_cmview_f *y);
void orc_rcfftmop_f(const orc_fftm_f *p, const orc_mview_f *x, const orc_cmview_f *z);
void orc_crfftmop_f(const orc_fftm_f *p, const orc_cmview_f *z, const orc_mview_f *x);
void orc_ccfftmop_d(const orc_fftm_d *p, const orc_cmview_d *x, const orc_cmview_d *y);
void orc_ccfftmip_d(const orc_fftm_d *p, const orc_cmview_d *y);
void orc_rcfftmop_d(const orc_fftm_d *p, const orc_mview_d *x, const orc_cmview_d *z);
void orc_crfftmop_d(const orc_fftm_d *p, const orc_cmview_d *z, const orc_mview_d *x);

/* Factorisation of c_VSIP_src/VI_nuV.h:22-136: returns the number of stages. */
unsigned long orc_factor(unsigned long N, unsigned long *pn, unsigned long *p0,
                         unsigned long *pF);
/* Digit reversal of c_VSIP_src/VI_jofk.h:21-48. */
unsigned long orc_jofk(unsigned long k, const unsigned long *pn, const unsigned long *p0,
                       unsigned long pF, unsigned long nstage);

/* Seeded synthetic inputs shared by tests and bench: SplitMix64 of
 * (seed, index) -> 53-bit uniform -> U[-1,1) or N(0,1) (Box-Muller, double),
 * rounded to the destination type.  dist 0 = U[-1,1), 1 = N(0,1). */
void orc_fill_f(float *dst, unsigned long n, unsigned long long seed, int dist);
void orc_fill_d(double *dst, unsigned long n, unsigned long long seed, int dist);

/* Run a ccfftmop_f over `rows` dense rows of length N split across `threads`
 * pthreads, each with its own plan on a disjoint slab (plans are not
 * reentrant).  Used for the all-cores CPU baseline.  Returns 0 on success. */
int orc_ccfftmop_rows_mt_f(unsigned long rows, unsigned long N, int dir, float scale,
                           const float *x, float *y, int threads);
int orc_ccfftmop_rows_mt_d(unsigned long rows, unsigned long N, int dir, double scale,
                           const double *x, double *y, int threads);

#ifdef __cplusplus
}
#endif
#endif
