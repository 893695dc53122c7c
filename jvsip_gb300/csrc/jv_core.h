// jv_core.h -- internal interfaces of the GB300 fftm library: error state,
// device context, device memory pool, block residency table, plan object and
// the kernel launch descriptors shared by the host runtime and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "vsip_layout.h"

namespace jv {

// ------------------------------------------------------------------ errors
// Error codes returned by jvsip_gpu_last_error().
enum Err {
    OK = 0,
    E_NODEVICE = 1,    // no usable CUDA device
    E_ALLOC = 2,       // device or pinned allocation failed
    E_ARG = 3,         // invalid plan / view / length
    E_CUDA = 4,        // a CUDA runtime call failed
    E_UNSUPPORTED = 5, // combination this library does not handle
    E_DEVICE = 6       // a kernel reported a device-side status (bounded wait expired)
};
void set_error(int code, const std::string &msg);
bool cuda_ok(cudaError_t e, const char *what);   // records and returns false on error

// ------------------------------------------------------------------ device
struct Device {
    int id = -1;
    int sms = 0;
    size_t smem_optin = 0;     // max dynamic shared memory per block (opt-in)
    cudaStream_t stream = nullptr;  // library stream (all device work is ordered on it)
    cudaStream_t h2d = nullptr;     // staging copy streams for host-resident views
    cudaStream_t d2h = nullptr;
    cudaEvent_t ev[128];            // chunk events of the pipelined staging path
};
Device *device();   // lazily initialised; nullptr (and error recorded) when no GPU

// Kernel launches issued by this library (all kernels), for tools and benchmarks.
void count_launch(unsigned n = 1);

// ------------------------------------------------------------------ memory pool
// Caching device allocator: freed buffers are kept per exact size class and
// reused, so repeated calls do not cudaMalloc.  Thread-safe.
void *dmalloc(size_t bytes);
void dfree(void *p);
void pool_trim();

// ------------------------------------------------------------------ residency
// Device mirror of an admitted block.  For interleaved complex blocks `d` holds
// 2*size scalars; for split blocks `d` holds the real part and `d_im` the
// imaginary part; for real blocks `d` holds size*rstride scalars.
struct Mirror {
    void *d = nullptr;
    void *d_im = nullptr;
    size_t bytes = 0;          // bytes of each device array
    bool device_newer = false; // device written since the last host sync
};
Mirror *mirror_find(const void *block);           // nullptr when the block is not mirrored
Mirror *mirror_create(const void *block, size_t bytes, bool split);
void mirror_drop(const void *block);

// Pinned host arrays handed out by vsip_*blockcreate_* (freed with cudaFreeHost).
bool pinned_owned(const void *p);
void *host_alloc(size_t bytes);
void host_free(void *p);

// ------------------------------------------------------------------ views on the device
// A complex view in transform order: element n of vector v is at complex index
// off + v*vs + n*es of the arrays (re, im); scalar index = cst * complex index.
struct CView {
    void *re = nullptr, *im = nullptr;
    long cst = 2, off = 0, es = 1, vs = 0;
};
// A real view in transform order: element n of vector v at a[rst*(off + v*vs + n*es)].
struct RView {
    void *a = nullptr;
    long rst = 1, off = 0, es = 1, vs = 0;
};

enum Kind { K_C2C = 0, K_R2C = 1, K_C2R = 2 };
enum Prec { P_F32 = 0, P_F64 = 1 };

// One execution of a plan on resolved device views.
struct Job {
    int kind = K_C2C;
    int prec = P_F32;
    long N = 0;          // complex FFT length (R2C/C2R: the half length MN)
    long nvec = 0;       // number of transforms
    int inv = 0;         // 1: inverse direction (exp(+2 pi i nk/N))
    int has_scale = 0;
    double scale = 1.0;
    CView cin, cout;     // complex input / output
    RView rin, rout;     // real input (R2C) / output (C2R)
    int inplace = 0;     // input and output are the same storage
    const void *tw = nullptr;     // forward table exp(-2 pi i m/N), m < N, dtype complex
    const void *thalf = nullptr;  // R2C/C2R table exp(-+ i pi k/MN), k <= MN
    const void *twp = nullptr;    // per-pass twiddle tables of the specialised kernel (or null)
    const void *twg = nullptr;    // per-pass twiddle tables of the general kernel's schedule
    const void *pc = nullptr;     // per-pass constants of that schedule (PassConst)
    const void *twdd = nullptr;   // per-pass double-float twiddles of the FP64 form (or null)
    int npass = 0;
    int radix[40];
    int form = 0;        // JVSIP_FORM_* of the plan
    bool no_fast = false;      // JVSIP_GPU_NO_FAST at plan creation: general kernels only
    bool no_pipeline = false;  // JVSIP_GPU_NO_PIPELINE at plan creation: one staging copy each way
    int tuned_vpb = 0, tuned_emax = 0;  // the plan's tuned shared-memory kernel shape (0: automatic)
    int tma_columns = -1;      // JVSIP_GPU_TMA_COLUMNS at plan creation: 1 / 0 force TMA-staged
                               // column tiles on / off, -1 (unset) automatic
    // the steps of a long transform (shared-memory kernel, interleaved c2c only)
    int conj_in = -1, conj_out = -1;   // conjugate on load / store: -1 follows inv
    long nbatch = 1;                   // groups of nvec transforms along the grid's y
    long bvs_in = 0, bvs_out = 0;      // complex-element offset between groups
    const void *tw_lo = nullptr;       // output twiddle W^(g*k) of the first step, g = t*tw_ts +
    const void *tw_hi = nullptr;       //   group*tw_ys: tw_lo[m & tw_mask] * tw_hi[m >> tw_sh]
    unsigned tw_mask = 0, tw_sh = 0, tw_ts = 0, tw_ys = 0;
    struct LongPlan *lp = nullptr;     // the plan's long-transform decomposition (or null)
    // a pass of a large-radix Stockham transform of 2^k points (radix N):
    // Ns = product of the earlier radices (2^sp_lgns), input twiddle exponent
    // stride Nt/(Ns*N), sp_mask = Nt - 1
    unsigned sp_ns = 1, sp_lgns = 0, sp_twstride = 0, sp_mask = 0;
    // the k-omega pipeline (its own kernel instances): R2C rows tapered as they
    // are loaded -- real element n of transform t times taper_n[n*taper_n_st],
    // then times taper_t[t*taper_t_st], written back when taper_back -- and c2c
    // columns storing (gram_scale*|X|^2, Im X) with gram[t*gram_vs + k*gram_es]
    // += gram_scale*|X|^2
    const void *taper_n = nullptr, *taper_t = nullptr;
    long taper_n_st = 1, taper_t_st = 1;
    int taper_back = 0;
    void *gram = nullptr;
    long gram_es = 0, gram_vs = 0;
    double gram_scale = 1.0;
};

// A device-resident call of a plan captured into a CUDA graph: plans created
// with ntimes == 0 ("many times") capture the launch sequence of a call the
// second time they see its views and replay it afterwards.
struct CallGraph {
    Job key;                        // the resolved call
    cudaGraphExec_t exec = nullptr;
    unsigned kernels = 0;           // kernel launches the graph holds
    bool failed = false;            // capture was refused: run directly
};
void count_launch_undo(unsigned long long n);  // launches recorded by a capture did not run

// A transform of N = N1 * N2 points too long for one CTA, as two steps of the
// shared-memory kernel: A, N1 transforms of N2 points down the columns of x
// seen as an N2 x N1 row-major matrix (x[n1 + N1*n2]), each output element k2
// multiplied by W_N^(n1*k2) and stored as row n1 of an N1 x N2 scratch
// matrix; B, N2 transforms of N1 points down the scratch's columns, element
// k1 of column k2 stored at y[k2 + N2*k1].
struct LongPlan {
    long N1 = 0, N2 = 0;
    struct Plan *p1 = nullptr, *p2 = nullptr;  // c2c plans of N1 and N2 points (schedules, tables)
    // single vectors of 2^k points (f32): passes of radix sp_radix[i] (64..2048)
    // in the register-resident kernel's column tiles, plans of those lengths
    std::vector<long> sp_radix;
    std::vector<struct Plan *> sp_plans;
    void *d_lo = nullptr, *d_hi = nullptr;     // two-level table of W_N^m: lo[m & mask] * hi[m >> sh]
    unsigned mask = 0, sh = 0;
    void *scratch = nullptr;                   // nvec * N complex, allocated at the first call
    size_t scratch_bytes = 0;
};

// Shortest length run as two steps when a plan has fewer transforms than half
// the SMs (one CTA per transform would leave most of the GPU idle).
constexpr long kLongFewMin = 8192;
// Shortest length whose single-precision c2c columns (adjacent vectors) run as
// two steps whatever their count, unless the register-resident column tiles
// take the length (fast_step_len: powers of two up to 4096 and 1000).
// Measured on columns of 3000-7776 points (128-1024 of them): 1.1-1.7x the
// shared-memory kernel's column tiles; 8192-16384 points: 1.1-3.0x; below,
// mixed (2187 x 1024: 1.07x, 2560 x 1024: 0.91x, 2400 x 512: 0.70x).
constexpr long kColStepsMin = 3000;

// Kernel entry points (defined in the kernel translation units).
bool launch_smem_f32(const Job &j, cudaStream_t s);
bool launch_smem_f64(const Job &j, cudaStream_t s);
bool launch_smem_real_f32(const Job &j, cudaStream_t s);  // R2C / C2R instances
bool launch_smem_split_f32(const Job &j, cudaStream_t s); // c2c on split complex views (both sides)
bool launch_smem_split_f64(const Job &j, cudaStream_t s);
bool launch_komega_r2c_f32(const Job &j, cudaStream_t s); // tapered R2C rows (taper_* set)
bool launch_komega_power_f32(const Job &j, cudaStream_t s); // c2c columns accumulating power (gram set)
bool launch_smem_real_f64(const Job &j, cudaStream_t s);
bool launch_global_f32(const Job &j, cudaStream_t s);
bool launch_global_f64(const Job &j, cudaStream_t s);
bool launch_fast_f32(const Job &j, cudaStream_t s);   // specialised kernels; false when none fits
bool launch_fast_real_f32(const Job &j, cudaStream_t s);  // R2C / C2R rows on the specialised kernel
bool launch_fast_komega_r2c_f32(const Job &j, cudaStream_t s);    // k-omega tapered R2C rows (specialised kernel)
bool launch_fast_komega_power_f32(const Job &j, cudaStream_t s);  // k-omega power columns (specialised kernel)
std::vector<int> fast_radices(long N);                // radix list of the specialised kernel for N
bool fast_step_len(long N);                           // lengths the specialised kernel takes as long-transform steps
bool launch_fast_step_f32(const Job &j, cudaStream_t s);  // a long-transform step in column-tile mode (single group)
bool launch_fast_sp_f32(const Job &j, cudaStream_t s);    // a pass of a large-radix Stockham transform (sp_* set)
bool launch_split_f32(const Job &j, cudaStream_t s);  // precision form; false when the call does not qualify
bool launch_fast_dd(const Job &j, cudaStream_t s);    // FP64 form (double-float rows); false when it does not qualify
std::vector<int> dd_radices(long N);                  // radix list of the FP64 form for N (empty: none)
int split_status_check(cudaStream_t s);               // device status of the precision form (0 = clean)
// real long transforms: in-place Hermitian split of Z on an interleaved view,
// C2R un-split into dense conjugated Y, and the final store of dense conjugated y
bool launch_r2c_pairs_f32(void *z, long es, long vs, long N, long nvec, int has_scale, double scale,
                          const void *thalf, cudaStream_t s);
bool launch_r2c_pairs_f64(void *z, long es, long vs, long N, long nvec, int has_scale, double scale,
                          const void *thalf, cudaStream_t s);
bool launch_c2r_unsplit_f32(const Job &j, void *ydst, cudaStream_t s);
bool launch_c2r_unsplit_f64(const Job &j, void *ydst, cudaStream_t s);
bool launch_c2r_unpack_f32(const Job &j, const void *y, cudaStream_t s);
bool launch_c2r_unpack_f64(const Job &j, const void *y, cudaStream_t s);
int *kernel_status();                                 // device word a kernel sets when a bounded wait expired
bool test_wait_expiry();                              // test hook: TMA-staged tiles make their wait expire
int kernel_status_check(cudaStream_t s);              // reads and clears it (0 = clean)

// Capacity queries used by the dispatcher.
long smem_max_len(int prec, int kind);   // largest N the shared-memory kernel takes

// ------------------------------------------------------------------ plans
struct Plan {
    int type = JV_CCFFTOP;    // JV_CCFFTOP / CCFFTIP / RCFFTOP / CRFFTOP
    int prec = P_F32;
    long M = 0, N = 0, MN = 0, mN = 0;
    int major = 0;            // 0 = VSIP_ROW, 1 = VSIP_COL
    int dir = -1;
    double scale = 1.0;
    unsigned ntimes = 0;
    int hint = 0;
    int form = 0;             // JVSIP_FORM_*
    bool no_fast = false;     // environment switches read once at creation
    bool no_pipeline = false;
    int tma_columns = -1;
    int tuned_vpb = 0;        // tuned transforms per CTA of the shared-memory kernel (0: heuristic)
    int tuned_emax = 0;       // tuned complex values per thread and pass, 8 or 16 (0: automatic)
    bool tuned = false;       // the autotuner's entry for (MN, precision, stride class) was applied
    std::vector<int> radix;   // pass radices of the device kernels (product = MN)
    bool smooth = true;       // every radix is one of the built-in codelets
    void *d_tw = nullptr;     // forward twiddles, MN entries
    void *d_thalf = nullptr;  // half-angle table, MN+1 entries (real transforms)
    void *d_twp = nullptr;    // per-pass [r][m] twiddle tables of the specialised kernel
    void *d_twg = nullptr;    // per-pass [r][m] twiddle tables of the general kernel's schedule
    void *d_pc = nullptr;     // per-pass constants of that schedule (PassConst, one per pass)
    void *d_twdd = nullptr;   // per-pass double-float tables of the FP64 form (built by setform_d)
    std::vector<unsigned long> jofk;  // reference digit-reversal map (kept for parity checks)
    std::vector<CallGraph> graphs;    // captured calls (ntimes == 0), most recent last
    bool single = false;      // a single-FFT plan (vsip_fft_*: one row, vector views)
    LongPlan *lp = nullptr;   // two-step decomposition when MN is too long for one CTA
    std::mutex mu;            // the plan is used by one call at a time
};

Plan *plan_of(const void *vsip_plan);   // ext_fftm_obj of a vsip_fftm_* (nullptr if bad)
Plan *plan_of_v(const void *vsip_plan); // ext_fft_obj of a vsip_fft_* (nullptr if bad)
// A single-precision c2c call on views of admitted interleaved blocks, enqueued
// on `st` with no host synchronisation (the batching form's route for long
// columns); with `prepare` only the plan's long-transform scratch is made
// ready and nothing is launched.  False (error set) when it cannot run so.
bool enqueue_resident_c2c_f(Plan *p, const vsip_cmview_f *x, const vsip_cmview_f *y, cudaStream_t st, bool prepare);
// true when such a call of plan p on these views runs as the long columns' two steps
bool resident_long_columns_f(Plan *p, const vsip_cmview_f *x, const vsip_cmview_f *y);

// factorisation of the reference (c_VSIP_src/VI_nuV.h:22-136); returns the stage count
unsigned long ref_factor(unsigned long N, unsigned long *pn, unsigned long *p0, unsigned long *pF);
// Constants of one pass of the general kernel's schedule: NR = N/R, the
// multiply-high magic of NR and of Ns (product of the earlier radices), Ns.
struct PassConst {
    unsigned NR, mNR, Ns, mNs;
};
// floor(x / d) == __umulhi(x, m) for x * d < 2^32 with m = ceil(2^32 / d); 0 encodes d = 1
inline unsigned magic_host(unsigned long d) { return d <= 1 ? 0u : (unsigned)(0xFFFFFFFFul / d + 1ul); }
// Butterflies a thread keeps per radix-R pass of the general kernel sized for
// EMAX points: ceil(EMAX/R) for the prime-power codelets (R <= 8), one (or
// EMAX/R) for the composite ones, whose registers are already R points.
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr int pass_k(int EMAX, int R) { return R <= 8 ? (EMAX + R - 1) / R : (EMAX >= R ? EMAX / R : 1); }
// Radix codelets of the general kernel, in the order of its pass loops.
constexpr int kRadices = 13;
constexpr int kRadixList[kRadices] = {16, 15, 14, 12, 10, 9, 8, 7, 6, 5, 4, 3, 2};
// ------------------------------------------------------------------ autotuner
// A tuned configuration of the c2c path for one (length, precision, stride
// class): residency (0: the register-resident kernel where an instance exists,
// 1: the shared-memory kernel), the shared-memory kernel's pass schedule,
// transforms per CTA (0: heuristic) and complex values a thread keeps per pass
// (8 or 16; 0: automatic).  Stride class 0: transforms along contiguous rows
// (VSIP_ROW plans), 1: adjacent transforms (VSIP_COL plans).
struct PlainTune {
    int res = 0;
    std::vector<int> radix;
    int vpb = 0;
    int emax = 0;
};
bool plain_tuned(long N, int prec, int cls, PlainTune *out);  // the forced or cached entry
void plain_tune_force(const PlainTune *t);  // this thread's plans use t instead of the cache (nullptr: off)
// Schedules of the shared-memory kernel for N (2^a 3^b 5^c 7^d): the default
// (fewest passes, largest radices first) first, then the other decompositions
// into codelet radices with at most one pass more, each largest first (the
// kernel runs its codelets in that order); at most `limit` of them.
std::vector<std::vector<int>> schedule_candidates(long N, long maxt, size_t limit);
bool schedule_valid(const std::vector<int> &r, long N, long maxt);

inline bool gpass_codelet_host(int R) {
    for (int i = 0; i < kRadices; i++)
        if (kRadixList[i] == R) return true;
    return false;
}
// device pass radices for length N: for 2^a 3^b 5^c 7^d the fewest passes of
// the codelets above (largest first), else radix 8/4/2, 3, 5, 7, then any other prime
std::vector<int> pass_radices(long N, bool *smooth, long maxt);  // maxt: threads per CTA of the shared-memory kernel

}  // namespace jv
