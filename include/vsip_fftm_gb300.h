/*
 * vsip_fftm_gb300.h -- C ABI of the GB300 (sm_103a) multiple-FFT library.
 *
 * The library exports the VSIPL 1.3 multiple-FFT calls with the exact
 * prototypes of the jvsip reference (c_VSIP_src/vsip.h), so an application
 * built against the reference header links this library ahead of libvsip.a
 * and its fftm calls run on the GPU while every other VSIPL call still
 * resolves to the reference.  Each declaration cites the reference prototype
 * it replaces as c_VSIP_src/vsip.h:<line>.
 *
 * The header is C89/C99 clean.  When the reference's vsip.h has already been
 * included (its guard _VSIP_H is defined) the VSIPL types come from there;
 * otherwise this header declares the subset the fftm calls use, with the same
 * names, underlying types and enumerator values as c_VSIP_src/vsip.h:124-208,
 * 277-278, so that objects cross the two libraries unchanged.
 *
 * Residency: a block admitted through vsip_cblockadmit_* / vsip_blockadmit_*
 * of this library gets a device mirror (uploaded when update is true).  fftm
 * calls on views of admitted blocks run device to device and leave the result
 * on the device until the block is released (downloaded when update is true)
 * or synchronised with jvsip_cblocksync_* / jvsip_blocksync_*.  Views of
 * blocks that are not admitted (VSIPL-created blocks, or user blocks used
 * without admission) are staged through the device inside each call, so the
 * host data is up to date when the call returns.
 *
 * Errors: create calls return NULL on any failure (bad length, allocation
 * failure, no CUDA device) and free what they had allocated, as the reference
 * does (c_VSIP_src/VI_ccfftmop_create_f_def.h:34,50-55).  Execution calls are
 * void as in the reference; a failure is recorded for jvsip_gpu_last_error()
 * and never aborts the process.
 */
#ifndef VSIP_FFTM_GB300_H
#define VSIP_FFTM_GB300_H 1

#include <stddef.h>

#ifndef _VSIP_H
/* ---- VSIPL scalar, enum and opaque handle types (c_VSIP_src/vsip.h:124-208) ---- */
typedef signed int        vsip_scalar_bl;
typedef vsip_scalar_bl    vsip_bool;
typedef float             vsip_scalar_f;
typedef double            vsip_scalar_d;
typedef unsigned long int vsip_scalar_vi;
typedef vsip_scalar_vi    vsip_offset;
typedef vsip_scalar_vi    vsip_length;
typedef vsip_scalar_vi    vsip_index;
typedef signed long int   vsip_stride;
typedef struct { vsip_scalar_vi r, c; } vsip_scalar_mi;
typedef struct { vsip_scalar_d r, i; } vsip_cscalar_d;
typedef struct { vsip_scalar_f r, i; } vsip_cscalar_f;
typedef enum { VSIP_MEM_NONE = 0, VSIP_MEM_RDONLY = 1, VSIP_MEM_CONST = 2,
               VSIP_MEM_SHARED = 3, VSIP_MEM_SHARED_RDONLY = 4,
               VSIP_MEM_SHARED_CONST = 5 } vsip_memory_hint;
typedef enum { VSIP_ROW = 0, VSIP_COL = 1 } vsip_major;
typedef enum { VSIP_FFT_FWD = -1, VSIP_FFT_INV = +1 } vsip_fft_dir;
typedef enum { VSIP_FFT_IP = 0, VSIP_FFT_OP = 1 } vsip_fft_place;
typedef enum { VSIP_ALG_SPACE = 0, VSIP_ALG_TIME = 1, VSIP_ALG_NOISE = 2 } vsip_alg_hint;
typedef struct vsip_blockattributes_f  vsip_block_f;
typedef struct vsip_blockattributes_d  vsip_block_d;
typedef struct vsip_cblockattributes_f vsip_cblock_f;
typedef struct vsip_cblockattributes_d vsip_cblock_d;
typedef struct vsip_mviewattributes_f  vsip_mview_f;
typedef struct vsip_mviewattributes_d  vsip_mview_d;
typedef struct vsip_cmviewattributes_f vsip_cmview_f;
typedef struct vsip_cmviewattributes_d vsip_cmview_d;
typedef struct vsip_fftmattributes_f   vsip_fftm_f;
typedef struct vsip_fftmattributes_d   vsip_fftm_d;
/* c_VSIP_src/vsip.h:174-175, 187-188, 205-206 */
typedef struct vsip_vviewattributes_f  vsip_vview_f;
typedef struct vsip_vviewattributes_d  vsip_vview_d;
typedef struct vsip_cvviewattributes_f vsip_cvview_f;
typedef struct vsip_cvviewattributes_d vsip_cvview_d;
typedef struct vsip_fftattributes_f    vsip_fft_f;
typedef struct vsip_fftattributes_d    vsip_fft_d;
/* c_VSIP_src/vsip.h:275-276 */
typedef struct { vsip_scalar_vi input; vsip_scalar_vi output; vsip_fft_place place;
                 vsip_scalar_d scale; vsip_fft_dir dir; } vsip_fft_attr_d;
typedef struct { vsip_scalar_vi input; vsip_scalar_vi output; vsip_fft_place place;
                 vsip_scalar_f scale; vsip_fft_dir dir; } vsip_fft_attr_f;
/* c_VSIP_src/vsip.h:277-278 */
typedef struct { vsip_scalar_mi input; vsip_scalar_mi output; vsip_fft_place place;
                 vsip_scalar_d scale; vsip_fft_dir dir; vsip_major major; } vsip_fftm_attr_d;
typedef struct { vsip_scalar_mi input; vsip_scalar_mi output; vsip_fft_place place;
                 vsip_scalar_f scale; vsip_fft_dir dir; vsip_major major; } vsip_fftm_attr_f;
#endif /* _VSIP_H */

#ifdef __cplusplus
extern "C" {
#endif

/* ======================= multiple-FFT plans ======================= */
/* c_VSIP_src/vsip.h:1814 -- c_VSIP_src/VI_ccfftmop_create_f_def.h:23-88 */
vsip_fftm_f *vsip_ccfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale,
                                    vsip_fft_dir dir, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1813 -- c_VSIP_src/VI_ccfftmip_create_f_def.h:23-86 */
vsip_fftm_f *vsip_ccfftmip_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale,
                                    vsip_fft_dir dir, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1816 -- c_VSIP_src/VI_rcfftmop_create_f_def.h:26-99 */
vsip_fftm_f *vsip_rcfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1815 -- c_VSIP_src/VI_crfftmop_create_f_def.h:24-96 */
vsip_fftm_f *vsip_crfftmop_create_f(vsip_length M, vsip_length N, vsip_scalar_f scale,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1810 */
vsip_fftm_d *vsip_ccfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale,
                                    vsip_fft_dir dir, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1809 */
vsip_fftm_d *vsip_ccfftmip_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale,
                                    vsip_fft_dir dir, vsip_major major,
                                    unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1812 */
vsip_fftm_d *vsip_rcfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1811 */
vsip_fftm_d *vsip_crfftmop_create_d(vsip_length M, vsip_length N, vsip_scalar_d scale,
                                    vsip_major major, unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:426 -- c_VSIP_src/vsip_fftm_destroy_f.c:20-40 (NULL-safe, returns 0) */
int vsip_fftm_destroy_f(vsip_fftm_f *plan);
/* c_VSIP_src/vsip.h:425 */
int vsip_fftm_destroy_d(vsip_fftm_d *plan);
/* c_VSIP_src/vsip.h:947 -- c_VSIP_src/vsip_fftm_getattr_f.c:18-69 */
void vsip_fftm_getattr_f(const vsip_fftm_f *plan, vsip_fftm_attr_f *attr);
/* c_VSIP_src/vsip.h:946 */
void vsip_fftm_getattr_d(const vsip_fftm_d *plan, vsip_fftm_attr_d *attr);

/* ======================= multiple-FFT execution ======================= */
/* c_VSIP_src/vsip.h:717 -- c_VSIP_src/VI_ccfftmop_f_def.h:20-29 (x may alias y) */
void vsip_ccfftmop_f(const vsip_fftm_f *plan, const vsip_cmview_f *x, const vsip_cmview_f *y);
/* c_VSIP_src/vsip.h:715 -- c_VSIP_src/VI_ccfftmip_f_def.h:17-23 */
void vsip_ccfftmip_f(const vsip_fftm_f *plan, const vsip_cmview_f *xy);
/* c_VSIP_src/vsip.h:1184 -- c_VSIP_src/VI_rcfftmop_f_def.h:24-120 */
void vsip_rcfftmop_f(const vsip_fftm_f *plan, const vsip_mview_f *x, const vsip_cmview_f *y);
/* c_VSIP_src/vsip.h:827 -- c_VSIP_src/VI_crfftmop_f_def.h:25-126 */
void vsip_crfftmop_f(const vsip_fftm_f *plan, const vsip_cmview_f *x, const vsip_mview_f *y);
/* c_VSIP_src/vsip.h:716 */
void vsip_ccfftmop_d(const vsip_fftm_d *plan, const vsip_cmview_d *x, const vsip_cmview_d *y);
/* c_VSIP_src/vsip.h:714 */
void vsip_ccfftmip_d(const vsip_fftm_d *plan, const vsip_cmview_d *xy);
/* c_VSIP_src/vsip.h:1183 */
void vsip_rcfftmop_d(const vsip_fftm_d *plan, const vsip_mview_d *x, const vsip_cmview_d *y);
/* c_VSIP_src/vsip.h:826 */
void vsip_crfftmop_d(const vsip_fftm_d *plan, const vsip_cmview_d *x, const vsip_mview_d *y);

/* ======================= single-FFT plans (vectors) ======================= */
/* A single FFT is the one-row case of the multiple FFT: the same device plan,
 * kernels, residency rules and error behaviour, with vector views in place of
 * matrix views.  For rcfftop / crfftop plans N is the real length and the
 * plan keeps N/2 (c_VSIP_src/VI_rcfftop_create_f_def.h:35). */
/* c_VSIP_src/vsip.h:1806 -- c_VSIP_src/VI_ccfftop_create_f_def.h:24-81 */
vsip_fft_f *vsip_ccfftop_create_f(vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir,
                                  unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1805 */
vsip_fft_f *vsip_ccfftip_create_f(vsip_length N, vsip_scalar_f scale, vsip_fft_dir dir,
                                  unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1808 -- c_VSIP_src/VI_rcfftop_create_f_def.h:26-92 */
vsip_fft_f *vsip_rcfftop_create_f(vsip_length N, vsip_scalar_f scale, unsigned int ntimes,
                                  vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1807 -- c_VSIP_src/VI_crfftop_create_f_def.h:23-89 */
vsip_fft_f *vsip_crfftop_create_f(vsip_length N, vsip_scalar_f scale, unsigned int ntimes,
                                  vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1802 */
vsip_fft_d *vsip_ccfftop_create_d(vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir,
                                  unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1801 */
vsip_fft_d *vsip_ccfftip_create_d(vsip_length N, vsip_scalar_d scale, vsip_fft_dir dir,
                                  unsigned int ntimes, vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1804 */
vsip_fft_d *vsip_rcfftop_create_d(vsip_length N, vsip_scalar_d scale, unsigned int ntimes,
                                  vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:1803 */
vsip_fft_d *vsip_crfftop_create_d(vsip_length N, vsip_scalar_d scale, unsigned int ntimes,
                                  vsip_alg_hint hint);
/* c_VSIP_src/vsip.h:424 (NULL-safe, returns 0) */
int vsip_fft_destroy_f(vsip_fft_f *plan);
/* c_VSIP_src/vsip.h:423 */
int vsip_fft_destroy_d(vsip_fft_d *plan);
/* c_VSIP_src/vsip.h:945 -- c_VSIP_src/vsip_fft_getattr_f.c:18-57 */
void vsip_fft_getattr_f(const vsip_fft_f *plan, vsip_fft_attr_f *attr);
/* c_VSIP_src/vsip.h:944 */
void vsip_fft_getattr_d(const vsip_fft_d *plan, vsip_fft_attr_d *attr);
/* c_VSIP_src/vsip.h:719 -- c_VSIP_src/VI_ccfftop_f_def.h:19-28 (x may alias y) */
void vsip_ccfftop_f(const vsip_fft_f *plan, const vsip_cvview_f *x, const vsip_cvview_f *y);
/* c_VSIP_src/vsip.h:713 */
void vsip_ccfftip_f(const vsip_fft_f *plan, const vsip_cvview_f *xy);
/* c_VSIP_src/vsip.h:1186 -- c_VSIP_src/VI_rcfftop_f_def.h:22-101 */
void vsip_rcfftop_f(const vsip_fft_f *plan, const vsip_vview_f *x, const vsip_cvview_f *y);
/* c_VSIP_src/vsip.h:829 -- c_VSIP_src/VI_crfftop_f_def.h:20-87 */
void vsip_crfftop_f(const vsip_fft_f *plan, const vsip_cvview_f *x, const vsip_vview_f *y);
/* c_VSIP_src/vsip.h:718 */
void vsip_ccfftop_d(const vsip_fft_d *plan, const vsip_cvview_d *x, const vsip_cvview_d *y);
/* c_VSIP_src/vsip.h:712 */
void vsip_ccfftip_d(const vsip_fft_d *plan, const vsip_cvview_d *xy);
/* c_VSIP_src/vsip.h:1185 */
void vsip_rcfftop_d(const vsip_fft_d *plan, const vsip_vview_d *x, const vsip_cvview_d *y);
/* c_VSIP_src/vsip.h:828 */
void vsip_crfftop_d(const vsip_fft_d *plan, const vsip_cvview_d *x, const vsip_vview_d *y);

/* ======================= blocks and views (the fftm boundary) ======================= */
/* c_VSIP_src/vsip.h:432, 427 -- no-ops in the reference; here they also set up / tear down the device */
int vsip_init(void *ptr);
int vsip_finalize(void *ptr);
/* c_VSIP_src/vsip.h:356 -- c_VSIP_src/VI_cblockbind_f_di.h (Ip NULL => interleaved) */
vsip_cblock_f *vsip_cblockbind_f(vsip_scalar_f *const Rp, vsip_scalar_f *const Ip,
                                 vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:348 */
vsip_cblock_d *vsip_cblockbind_d(vsip_scalar_d *const Rp, vsip_scalar_d *const Ip,
                                 vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:357 -- c_VSIP_src/vsip_cblockcreate_f.c (interleaved storage) */
vsip_cblock_f *vsip_cblockcreate_f(vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:349 */
vsip_cblock_d *vsip_cblockcreate_d(vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:372 -- c_VSIP_src/VI_cblockadmit_f_di.h:16-29; plus device mirror */
int vsip_cblockadmit_f(vsip_cblock_f *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:371 */
int vsip_cblockadmit_d(vsip_cblock_d *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:711 -- c_VSIP_src/VI_cblockrelease_f_di.h:16-34; plus download/free of the mirror */
void vsip_cblockrelease_f(vsip_cblock_f *b, vsip_scalar_bl update,
                          vsip_scalar_f **Rp, vsip_scalar_f **Ip);
/* c_VSIP_src/vsip.h:710 */
void vsip_cblockrelease_d(vsip_cblock_d *b, vsip_scalar_bl update,
                          vsip_scalar_d **Rp, vsip_scalar_d **Ip);
/* c_VSIP_src/vsip.h:705 -- c_VSIP_src/VI_cblockdestroy_f_di.h; plus freeing the mirror */
void vsip_cblockdestroy_f(vsip_cblock_f *b);
/* c_VSIP_src/vsip.h:704 */
void vsip_cblockdestroy_d(vsip_cblock_d *b);
/* c_VSIP_src/vsip.h:300 -- c_VSIP_src/vsip_blockbind_f.c */
vsip_block_f *vsip_blockbind_f(vsip_scalar_f *const p, vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:292 */
vsip_block_d *vsip_blockbind_d(vsip_scalar_d *const p, vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:301 -- c_VSIP_src/VI_blockcreate_f.h */
vsip_block_f *vsip_blockcreate_f(vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:293 */
vsip_block_d *vsip_blockcreate_d(vsip_length N, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:364 -- c_VSIP_src/vsip_blockadmit_f.c; plus device mirror */
int vsip_blockadmit_f(vsip_block_f *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:363 */
int vsip_blockadmit_d(vsip_block_d *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:1835 -- c_VSIP_src/vsip_blockrelease_f.c; plus download/free of the mirror */
vsip_scalar_f *vsip_blockrelease_f(vsip_block_f *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:1832 */
vsip_scalar_d *vsip_blockrelease_d(vsip_block_d *b, vsip_scalar_bl update);
/* c_VSIP_src/vsip.h:697 -- c_VSIP_src/vsip_blockdestroy_f.c */
void vsip_blockdestroy_f(vsip_block_f *b);
/* c_VSIP_src/vsip.h:696 */
void vsip_blockdestroy_d(vsip_block_d *b);
/* c_VSIP_src/vsip.h:455 -- c_VSIP_src/vsip_cmbind_f.c */
vsip_cmview_f *vsip_cmbind_f(const vsip_cblock_f *b, vsip_offset o, vsip_stride col_stride,
                             vsip_length col_length, vsip_stride row_stride,
                             vsip_length row_length);
/* c_VSIP_src/vsip.h:454 */
vsip_cmview_d *vsip_cmbind_d(const vsip_cblock_d *b, vsip_offset o, vsip_stride col_stride,
                             vsip_length col_length, vsip_stride row_stride,
                             vsip_length row_length);
/* c_VSIP_src/vsip.h:457 -- c_VSIP_src/vsip_mbind_f.c */
vsip_mview_f *vsip_mbind_f(const vsip_block_f *b, vsip_offset o, vsip_stride col_stride,
                           vsip_length col_length, vsip_stride row_stride,
                           vsip_length row_length);
/* c_VSIP_src/vsip.h:456 */
vsip_mview_d *vsip_mbind_d(const vsip_block_d *b, vsip_offset o, vsip_stride col_stride,
                           vsip_length col_length, vsip_stride row_stride,
                           vsip_length row_length);
/* c_VSIP_src/vsip.h:495 -- c_VSIP_src/vsip_cmcreate_f.c */
vsip_cmview_f *vsip_cmcreate_f(vsip_length M, vsip_length N, vsip_major major, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:494 */
vsip_cmview_d *vsip_cmcreate_d(vsip_length M, vsip_length N, vsip_major major, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:493 */
vsip_mview_f *vsip_mcreate_f(vsip_length M, vsip_length N, vsip_major major, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:492 */
vsip_mview_d *vsip_mcreate_d(vsip_length M, vsip_length N, vsip_major major, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:358 */
vsip_cblock_f *vsip_cmdestroy_f(vsip_cmview_f *v);
/* c_VSIP_src/vsip.h:350 */
vsip_cblock_d *vsip_cmdestroy_d(vsip_cmview_d *v);
/* c_VSIP_src/vsip.h:302 */
vsip_block_f *vsip_mdestroy_f(vsip_mview_f *v);
/* c_VSIP_src/vsip.h:294 */
vsip_block_d *vsip_mdestroy_d(vsip_mview_d *v);
/* c_VSIP_src/vsip.h:745 */
void vsip_cmalldestroy_f(vsip_cmview_f *v);
/* c_VSIP_src/vsip.h:744 */
void vsip_cmalldestroy_d(vsip_cmview_d *v);
/* c_VSIP_src/vsip.h:967 */
void vsip_malldestroy_f(vsip_mview_f *v);
/* c_VSIP_src/vsip.h:966 */
void vsip_malldestroy_d(vsip_mview_d *v);
/* c_VSIP_src/vsip.h:514 -- c_VSIP_src/vsip_cvbind_f.c */
vsip_cvview_f *vsip_cvbind_f(const vsip_cblock_f *b, vsip_offset o, vsip_stride s, vsip_length n);
/* c_VSIP_src/vsip.h:517 */
vsip_cvview_d *vsip_cvbind_d(const vsip_cblock_d *b, vsip_offset o, vsip_stride s, vsip_length n);
/* c_VSIP_src/vsip.h:491 -- c_VSIP_src/vsip_vbind_f.c */
vsip_vview_f *vsip_vbind_f(const vsip_block_f *b, vsip_offset o, vsip_stride s, vsip_length n);
/* c_VSIP_src/vsip.h:503 */
vsip_vview_d *vsip_vbind_d(const vsip_block_d *b, vsip_offset o, vsip_stride s, vsip_length n);
/* c_VSIP_src/vsip.h:512 */
vsip_cvview_f *vsip_cvcreate_f(vsip_length n, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:515 */
vsip_cvview_d *vsip_cvcreate_d(vsip_length n, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:488 */
vsip_vview_f *vsip_vcreate_f(vsip_length n, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:501 */
vsip_vview_d *vsip_vcreate_d(vsip_length n, vsip_memory_hint h);
/* c_VSIP_src/vsip.h:360 */
vsip_cblock_f *vsip_cvdestroy_f(vsip_cvview_f *v);
/* c_VSIP_src/vsip.h:352 */
vsip_cblock_d *vsip_cvdestroy_d(vsip_cvview_d *v);
/* c_VSIP_src/vsip.h:304 */
vsip_block_f *vsip_vdestroy_f(vsip_vview_f *v);
/* c_VSIP_src/vsip.h:296 */
vsip_block_d *vsip_vdestroy_d(vsip_vview_d *v);
/* c_VSIP_src/vsip.h:865 */
void vsip_cvalldestroy_f(vsip_cvview_f *v);
/* c_VSIP_src/vsip.h:864 */
void vsip_cvalldestroy_d(vsip_cvview_d *v);
/* c_VSIP_src/vsip.h:1292 */
void vsip_valldestroy_f(vsip_vview_f *v);
/* c_VSIP_src/vsip.h:1291 */
void vsip_valldestroy_d(vsip_vview_d *v);

/* ======================= extensions (not VSIPL) ======================= */
/* Status of the last failed call on this thread (0 = none) and its text;
 * jvsip_gpu_clear_error() resets it.  No reference counterpart: the reference
 * exec calls are void and unchecked (c_VSIP_src/vsip_crfftmop_f.c:14). */
int         jvsip_gpu_last_error(void);
const char *jvsip_gpu_last_error_string(void);
void        jvsip_gpu_clear_error(void);

/* Bring an admitted block's host array up to date with its device mirror
 * without releasing it.  Returns 0 on success. */
int jvsip_cblocksync_f(vsip_cblock_f *b);
int jvsip_cblocksync_d(vsip_cblock_d *b);
int jvsip_blocksync_f(vsip_block_f *b);
int jvsip_blocksync_d(vsip_block_d *b);

/* Execution form of a plan.  AUTO (default) picks the plain kernels;
 * SPLIT_BF16 / SPLIT_FP16 run radix-16/32 stages as tensor-core DFT products
 * with hi/lo operands and FP32 accumulation (c2c _f plans only). */
#define JVSIP_FORM_AUTO        0
#define JVSIP_FORM_PLAIN       1
#define JVSIP_FORM_SPLIT_BF16  2
#define JVSIP_FORM_SPLIT_FP16  3
int jvsip_fftm_setform_f(vsip_fftm_f *plan, int form);
int jvsip_fftm_getform_f(const vsip_fftm_f *plan);

/* FP64 form of a c2c _d plan of 64..8192 points (powers of two): contiguous
 * interleaved rows are transformed in double-float arithmetic (hi + lo
 * floats, 48 significant bits, each row shifted by a power of two so its
 * largest element lies in [1, 2)) on the FP32 pipes instead of the much
 * slower FP64 pipe; results agree with the plain form to about 1e-14
 * relative.  Other views and lengths keep the plain form.  Returns 0, or
 * JVSIP's error code (5: the plan's length or kind has no FP64 form). */
#define JVSIP_FORM_DF64        4
int jvsip_fftm_setform_d(vsip_fftm_d *plan, int form);
int jvsip_fftm_getform_d(const vsip_fftm_d *plan);

/* Batching form: run n independent c2c fftm calls (each plan with its own
 * input/output views; ccfftmop or ccfftmip plans) as one persistent launch fed
 * by a device work queue of (plan, row-tile) descriptors.  Equivalent to
 * calling vsip_ccfftmop_f / vsip_ccfftmip_f for i = 0..n-1 (in-place plans
 * use in[i]; out[i] is ignored).  Views must be of admitted blocks.
 * Returns 0 on success. */
int jvsip_fftm_batch_f(size_t n, const vsip_fftm_f *const plans[],
                       const vsip_cmview_f *const in[], const vsip_cmview_f *const out[]);

/* A captured batch: the descriptor queue is built and uploaded once and the
 * launch is recorded in a CUDA graph; jvsip_fftm_batch_run_f replays it.
 * The views' blocks must stay admitted (device addresses are baked in). */
typedef struct jvsip_fftm_batchplan_s jvsip_fftm_batchplan_f;
jvsip_fftm_batchplan_f *jvsip_fftm_batch_create_f(size_t n, const vsip_fftm_f *const plans[],
                                              const vsip_cmview_f *const in[],
                                              const vsip_cmview_f *const out[]);
int  jvsip_fftm_batch_run_f(jvsip_fftm_batchplan_f *batch);
int  jvsip_fftm_batch_destroy_f(jvsip_fftm_batchplan_f *batch);

/* The loop the batch replaces, run from C (no reference counterpart; the
 * reference's callers loop over vsip_ccfftmop_f, c_VSIP_src/VI_ccfftmop_f_def.h:20-29):
 * call i goes through vsip_ccfftmip_f(plans[i], in[i]) for in-place plans or
 * when out is NULL or out[i] is NULL, else vsip_ccfftmop_f(plans[i], in[i],
 * out[i]).  Returns 0, or the first call's error code (the remaining calls
 * are not made). */
int  jvsip_fftm_loop_f(size_t n, const vsip_fftm_f *const plans[],
                       const vsip_cmview_f *const in[], const vsip_cmview_f *const out[]);

/* Autotuner of the batching form: for each of the n lengths (2..16384;
 * vf = 1 for column transforms) time the batch kernel with each candidate
 * number of FFTs per tile and keep the fastest, in memory and in a versioned
 * cache file keyed by GPU name ($JVSIP_GPU_TUNE_CACHE, default
 * ~/.cache/jvsip_gb300/tune-v3.txt).  Untuned lengths use a heuristic.
 * Returns 0 on success; jvsip_fftm_autotune_entries() counts cached keys. */
int  jvsip_fftm_autotune_f(size_t n, const unsigned long *lengths, int vf);

/* Autotuner of the plain c2c calls (no reference counterpart; the reference's
 * radix order is fixed, c_VSIP_src/VI_nuV.h:22-136): for each of the n
 * single-precision lengths (2..16384 points of 2^a 3^b 5^c 7^d) and the stride
 * class cls (0: transforms along contiguous rows, as VSIP_ROW plans; 1:
 * adjacent transforms, as VSIP_COL plans) time the register-resident kernel
 * and the shared-memory kernel over radix schedules, transforms per CTA and
 * values per thread (threads per transform), and keep the fastest in the same
 * cache.  Plans created afterwards with that length, precision and major use
 * it.  Returns 0 on success. */
int  jvsip_fftm_autotune_plain_f(size_t n, const unsigned long *lengths, int cls);
/* The plain-call entry for (N, single precision, cls): residency (0:
 * register-resident kernel where one exists, 1: shared-memory kernel),
 * transforms per CTA (0: heuristic), values per thread and pass (0: automatic)
 * and up to maxr radices of the schedule; any pointer may be NULL.  Returns
 * the number of passes of the schedule, 0 when the length is untuned. */
int  jvsip_fftm_autotune_plain_entry_f(unsigned long N, int cls, int *res, int *vpb, int *emax, int *radices,
                                       int maxr);
long jvsip_fftm_autotune_entries(void);

/* Library / device information for tools (kernels compiled, SM count). */
const char *jvsip_gpu_build_info(void);
/* Device-side synchronisation: returns when all work this library queued has
 * finished; E_DEVICE (6) when a kernel's bounded wait expired since the last
 * synchronisation (the error is also recorded; the context stays usable). */
int jvsip_gpu_synchronize(void);
/* Test hook of the bounded device waits (no reference counterpart): while on
 * is nonzero, launches of the shared-memory kernel's TMA-staged column tiles
 * wait, after all their boxes have landed, on a barrier phase that nothing
 * completes, so that the wait runs out (short poll limit, no copy in flight)
 * and the kernel reports through the status word that the next
 * jvsip_gpu_synchronize returns as E_DEVICE.  Returns 0. */
int jvsip_gpu_test_wait_expiry(int on);
/* The CUDA stream (cudaStream_t, as void*) all of this library's device work
 * is ordered on; callers may record events on it or make their streams wait. */
void *jvsip_gpu_stream(void);
/* Number of kernels this library has launched since it was loaded. */
unsigned long jvsip_gpu_kernel_launches(void);
/* Plan introspection: the device pass radices (returns their count) and the
 * reference's digit-reversal map of the plan length (c_VSIP_src/VI_jofk.h),
 * kept for parity checks (returns the map length). */
int  jvsip_fftm_passes(const void *plan, int *radix, int cap);
long jvsip_fftm_jofk(const void *plan, unsigned long *out, long cap);
/* Number of calls of the plan held as captured CUDA graphs (no counterpart in
 * the reference).  A plan created with ntimes == 0 ("used many times")
 * captures the launch sequence of a device-resident call the second time it
 * sees the call's views and replays it afterwards (at most 8 per plan, the
 * oldest dropped); other plans and staged calls launch directly.  -1 for an
 * invalid plan. */
int  jvsip_fftm_graphs(const void *plan);

/* The k-omega power estimate of the reference's kw example
 * (examples/komegaExamples/kw_c/kw.c:8-26, komega()) in two launches instead
 * of seven library passes.  With Nsens x Nts real data, rcfftm a VSIP_ROW
 * rcfftmop _f plan (Nsens, Nts) and ccfftm a VSIP_COL ccfftm(ip|op) _f plan
 * (Nsens, Nts/2+1), it leaves exactly what kw.c's sequence
 *   vsip_vmmul_f(ts_taper, data, VSIP_ROW, data);
 *   vsip_vmmul_f(array_taper, data, VSIP_COL, data);
 *   vsip_rcfftmop_f(rcfftm, data, freq);  vsip_ccfftmip_f(ccfftm, freq);
 *   vsip_mcmagsq_f(freq, real(freq));     vsip_smmul_f(scale, real(freq), real(freq));
 *   vsip_madd_f(real(freq), gram, gram);
 * leaves: data tapered in place, freq = (scale*|X|^2, Im X), gram += scale*|X|^2
 * (tapers and power rounded in the reference's order; the transforms within
 * the fftm tolerance).  The R2C's first pass tapers the rows as it loads them
 * and the column transform's last pass stores the power and accumulates the
 * gram.  All blocks must be admitted; data rows of unit stride with an even
 * offset and pitch; freq interleaved.  Returns 0, or the error code also
 * recorded for jvsip_gpu_last_error(). */
int jvsip_komega_f(const vsip_fftm_f *rcfftm, const vsip_fftm_f *ccfftm,
                   const vsip_vview_f *ts_taper, const vsip_vview_f *array_taper,
                   const vsip_mview_f *data, const vsip_cmview_f *freq,
                   vsip_scalar_f scale, const vsip_mview_f *gram);

/* Complex-to-complex multiple FFT that allocates nothing (no counterpart in
 * the reference).  For callers that cannot allocate device memory when they
 * transform: real-time threads that must not block in the allocator,
 * applications whose device memory is fully reserved up front.  `plan` is a ccfftmop/ccfftmip _f plan made beforehand;
 * x and y are device pointers to interleaved complex float data (equal for an
 * in-place call).  For VSIP_ROW plans the mN transforms are rows of MN
 * contiguous points, x_pitch / y_pitch complex elements apart; for VSIP_COL
 * plans they are columns of a row-major matrix whose rows are x_pitch / y_pitch
 * apart.  The intermediate buffers come from a fixed 16 MiB array in device
 * memory that is part of the library (held on every GPU that loads it until
 * exit): mN*MN may not exceed 1048576 complex points, larger calls return an
 * error.  The array's address is looked up once, by the first call.  x and y
 * must be the same buffer
 * or not overlap.  All calls share the array and
 * it keeps the last call's contents; calls that overlap on the GPU race on it.
 * Work is queued on the library stream (jvsip_gpu_stream); returns 0 when it
 * was queued. */
int jvsip_ccfftm_noalloc_f(const vsip_fftm_f *plan, const void *x, long x_pitch, void *y, long y_pitch);

#ifdef __cplusplus
}
#endif
#endif /* VSIP_FFTM_GB300_H */
