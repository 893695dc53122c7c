/*
 * vsip_layout.h -- in-memory layout of the VSIPL objects this library reads
 * and creates.  The fields, their order and types are those of the jvsip
 * reference's default build (interleaved complex storage, neither
 * VSIP_ALWAYS_SPLIT nor VSIP_ALWAYS_INTERLEAVED defined), so blocks and views
 * made by either library can be handed to the other:
 *
 *   real block    c_VSIP_src/vsip_blockattributes_f.h:40-51
 *   complex block c_VSIP_src/vsip_cblockattributes_f.h:42-67
 *   real view     c_VSIP_src/vsip_mviewattributes_f.h:47-55
 *   complex view  c_VSIP_src/vsip_cmviewattributes_f.h:47-55
 *   plan          c_VSIP_src/vsip_fftmattributes_f.h:8-38
 *   vector views  c_VSIP_src/vsip_vviewattributes_f.h:46-52,
 *                 c_VSIP_src/vsip_cvviewattributes_f.h:45-51
 *   vector plan   c_VSIP_src/vsip_fftattributes_f.h:6-31
 *   constants     c_VSIP_src/VI.h:5-13
 *
 * The plan struct is opaque to callers; its first part mirrors the reference
 * plan so tools that peek at it see the same attribute fields, and
 * ext_fftm_obj (the reference's hook for an external FFT object,
 * vsip_fftmattributes_f.h:37) points to this library's device plan.
 */
#ifndef JV_VSIP_LAYOUT_H
#define JV_VSIP_LAYOUT_H

#include "../../include/vsip_fftm_gb300.h"

#define JV_VALID_OBJECT   0x5555
#define JV_FREED_OBJECT   0xAAAA
#define JV_RELEASED_BLOCK 0
#define JV_ADMITTED_BLOCK 1
#define JV_VSIPL_BLOCK    0
#define JV_USER_BLOCK     1
#define JV_DERIVED_BLOCK  2

#define JV_LAYOUT_BLOCK(SFX, T, CT)                                                      \
    struct vsip_blockattributes_##SFX {                                                   \
        vsip_cblock_##SFX *parent;  /* complex parent of a derived block          */      \
        T *array;                   /* data array                                 */      \
        int kind;                   /* VSIPL 0, user 1, derived 2                 */      \
        int admit;                  /* released 0, admitted 1                     */      \
        vsip_stride rstride;        /* scalar stride of one element               */      \
        vsip_length size;           /* elements                                   */      \
        int bindings;                                                                     \
        int markings;                                                                     \
        vsip_memory_hint hint;                                                            \
        vsip_scalar_bl update;                                                            \
    };                                                                                    \
    struct vsip_cblockattributes_##SFX {                                                  \
        vsip_block_##SFX *R, *I;    /* real / imaginary part blocks               */      \
        int kind;                                                                         \
        int admit;                                                                        \
        vsip_stride cstride;        /* 2 interleaved, 1 split                     */      \
        vsip_length size;           /* complex elements                           */      \
        int bindings;                                                                     \
        int markings;                                                                     \
        vsip_memory_hint hint;                                                            \
        CT a_scalar, a_zero, a_one, a_imag_one;                                           \
        vsip_scalar_bl update;                                                            \
    };                                                                                    \
    struct vsip_mviewattributes_##SFX {                                                   \
        vsip_block_##SFX *block;                                                          \
        vsip_offset offset;                                                               \
        vsip_stride row_stride;                                                           \
        vsip_length row_length;                                                           \
        vsip_stride col_stride;                                                           \
        vsip_length col_length;                                                           \
        int markings;                                                                     \
    };                                                                                    \
    struct vsip_cmviewattributes_##SFX {                                                  \
        vsip_cblock_##SFX *block;                                                         \
        vsip_offset offset;                                                               \
        vsip_stride row_stride;                                                           \
        vsip_length row_length;                                                           \
        vsip_stride col_stride;                                                           \
        vsip_length col_length;                                                           \
        int markings;                                                                     \
    };

JV_LAYOUT_BLOCK(f, vsip_scalar_f, vsip_cscalar_f)
JV_LAYOUT_BLOCK(d, vsip_scalar_d, vsip_cscalar_d)

/* Plan: transform kinds as c_VSIP_src/VI_ffttype.h. */
enum { JV_CCFFTOP = 0, JV_CCFFTIP = 1, JV_RCFFTOP = 2, JV_CRFFTOP = 3 };

/* The leading fields keep the reference's plan layout (pointer-sized slots for
 * its view/table pointers, which this library leaves NULL); the attributes the
 * reference's getattr reads are filled in with the reference's meaning. */
#define JV_LAYOUT_PLAN(SFX, T)                                                           \
    struct vsip_fftmattributes_##SFX {                                                    \
        void *wt, *temp, *index, *pn, *p0, *pF, *x;                                       \
        struct { void *block; vsip_offset offset; vsip_stride stride;                    \
                 vsip_length length; int markings; } xx;                                  \
        T *x_r, *x_i, *xp_r, *xp_i;                                                       \
        vsip_stride xst, yst, xpst, ypst;                                                 \
        T scale;                                                                          \
        vsip_length N;      /* row length                     */                          \
        vsip_length M;      /* column length                  */                          \
        vsip_length MN;     /* length along the major direction */                        \
        vsip_length mN;     /* number of transforms           */                          \
        vsip_major major;                                                                 \
        vsip_length length; /* number of factor stages        */                          \
        vsip_fft_dir d;                                                                   \
        int type;                                                                         \
        int dft;                                                                          \
        unsigned int ntimes;                                                              \
        vsip_alg_hint hint;                                                               \
        vsip_scalar_vi stage;                                                             \
        void *ext_fftm_obj; /* -> struct jv_plan (device plan) */                         \
    };

JV_LAYOUT_PLAN(f, vsip_scalar_f)
JV_LAYOUT_PLAN(d, vsip_scalar_d)

/* Vector views and the vector FFT plan (single transforms: one-row fftm). */
#define JV_LAYOUT_VECTOR(SFX, T)                                                         \
    struct vsip_vviewattributes_##SFX {                                                   \
        vsip_block_##SFX *block;                                                          \
        vsip_offset offset;                                                               \
        vsip_stride stride;                                                               \
        vsip_length length;                                                               \
        int markings;                                                                     \
    };                                                                                    \
    struct vsip_cvviewattributes_##SFX {                                                  \
        vsip_cblock_##SFX *block;                                                         \
        vsip_offset offset;                                                               \
        vsip_stride stride;                                                               \
        vsip_length length;                                                               \
        int markings;                                                                     \
    };                                                                                    \
    struct vsip_fftattributes_##SFX {                                                     \
        void *wt, *temp, *bit, *index, *pn, *p0, *pF, *x;                                 \
        T *x_r, *x_i, *xp_r, *xp_i;                                                       \
        vsip_stride xst, xpst;                                                            \
        T scale;                                                                          \
        vsip_length N;      /* length (R2C / C2R: the half length) */                     \
        vsip_length length; /* number of factor stages             */                     \
        vsip_fft_dir d;                                                                   \
        int type;                                                                         \
        int dft;                                                                          \
        unsigned int ntimes;                                                              \
        vsip_alg_hint hint;                                                               \
        vsip_scalar_vi stage;                                                             \
        void *ext_fft_obj;  /* -> struct jv_plan (device plan) */                         \
    };

JV_LAYOUT_VECTOR(f, vsip_scalar_f)
JV_LAYOUT_VECTOR(d, vsip_scalar_d)

#endif
