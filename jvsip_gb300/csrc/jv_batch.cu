// jv_batch.cu -- batching form: many independent c2c fftm calls (uneven
// lengths 2^a 3^b 5^c 7^d, uneven row counts, mixed directions and ROW/COL
// majors) in one launch per CTA-size class, fed by a device queue of tile
// descriptors.
//
// The host cuts every call into tiles of transforms (FFTs per tile from the
// autotuner's cache, or a heuristic), gives each tile the smallest CTA size
// (256, 512 or 1024 threads) whose threads cover its passes, and uploads one
// descriptor queue per size, largest tiles first.  One launch per size
// consumes its queue, one descriptor per CTA -- no CTA ever waits on another
// -- running the general kernel's fused c2c passes on each tile; the launches
// run side by side on forked streams.  Each CTA first asks L2 for the input
// of the descriptor one resident wave further down its queue (the CTA that
// will take this SM slot later), so later tiles' DRAM reads overlap earlier
// tiles' passes.  Columns of 8192 points or more (adjacent, more than one) go
// through the plain calls' two steps instead, on four more streams.  A
// captured batch (jvsip_fftm_batch_create_f) records the launches in a CUDA
// graph once; jvsip_fftm_batch_run_f replays it.
//
// No reference counterpart: VSIPL has no multi-plan call; the reference can
// only loop plan by plan (c_VSIP_src/VI_ccfftmop_f_def.h:20-29 per call).
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include <cooperative_groups.h>

#include "jv_launch.cuh"

namespace jv {

// one tile: nt transforms [v0, v0+nt) of one call
struct TileDesc {
    const float *in;    // interleaved views, complex index off + v*vs + n*es
    float *out;
    long in_off, in_es, in_vs;
    long out_off, out_es, out_vs;
    const float2 *twg;  // per-pass [r][m] tables of the call's plan
    const uint4 *pc;    // per-pass constants of the plan's schedule
    unsigned long long passes;  // pass counts per codelet (pass_count)
    unsigned mnt;       // multiply-high magic of nt
    long v0;
    int N, nt, ld;
    unsigned char inv, vec_fast, cls;  // cls: CTA-size class (index into kClassBT)
    int has_scale;
    float scale;
};

constexpr int BT = 1024;      // threads of the largest batch CTA
constexpr int BEMAX = 16;     // complex values a thread keeps per pass: tiles of <= 16384 points
// CTA-size classes: a tile runs in the smallest CTA whose threads cover every
// pass of it, so small tiles share an SM (4 x 256 or 2 x 512 threads at 64
// registers) instead of idling most of a 1024-thread CTA
constexpr int kClasses = 4;
constexpr int kClassBT[kClasses] = {256, 512, 1024, 1024};  // the last: column clusters
constexpr int kColClass = 3;

__device__ __forceinline__ void batch_tile(const TileDesc &d, float2 *s) {
    TileIO<float> io;
    io.in = reinterpret_cast<const float2 *>(d.in) + (d.in_off + d.v0 * d.in_vs);
    io.out = reinterpret_cast<float2 *>(d.out) + (d.out_off + d.v0 * d.out_vs);
    io.in_es = d.in_es;
    io.in_vs = d.in_vs;
    io.out_es = d.out_es;
    io.out_vs = d.out_vs;
    io.smask_in = io.smask_out = d.inv ? 0x80000000u : 0u;
    io.has_scale = d.has_scale != 0;
    io.scale = d.has_scale ? d.scale : 1.f;
    io.vf = io.vf_out = d.vec_fast != 0;
    io.mnt = d.mnt;
    io.tw_lo = io.tw_hi = nullptr;
    c2c_tile<float, BEMAX>(s, d.ld, d.nt, d.passes, d.twg, d.pc, io);
}

__device__ __forceinline__ void prefetch_l2_line(const void *p) {
    asm volatile("{\n\t.reg .u64 a;\n\tcvta.to.global.u64 a, %0;\n\tprefetch.global.L2 [a];\n\t}" :: "l"(p));
}

// Ask L2 for the input of tile d: one 128-byte line per thread and step.
// Transforms contiguous in memory (|es| = 1) go by 16-element segments of each
// transform, adjacent transforms (|vs| = 1) by 16-element segments of each
// point's row of transforms; other layouts are not prefetched.
__device__ __forceinline__ void prefetch_tile(const TileDesc &d, int tid, int nthr) {
    const float2 *base = reinterpret_cast<const float2 *>(d.in) + (d.in_off + d.v0 * d.in_vs);
    // every address is an element of the tile (the last line of a segment
    // is taken at its last element)
    if (d.in_es == 1) {
        const int L = (d.N + 15) >> 4, tot = L * d.nt;
        for (int i = tid; i < tot; i += nthr) {
            const int v = i / L, l = i - v * L;
            prefetch_l2_line(base + (long)v * d.in_vs + min(16 * l, d.N - 1));
        }
    } else if (d.in_vs == 1) {
        const int L = (d.nt + 15) >> 4, tot = L * d.N;
        for (int i = tid; i < tot; i += nthr) {
            const int n = i / L, l = i - n * L;
            prefetch_l2_line(base + (long)n * d.in_es + min(16 * l, d.nt - 1));
        }
    }
}

// One launch over the whole queue: CTA b takes descriptor b.  The queue is
// sorted largest tile first, so the hardware's in-order CTA dispatch hands the
// long tiles out first and the short ones fill the tail.  (A persistent
// variant -- each CTA looping over an atomic queue head -- was built and
// measured against ptxas: keeping the pass state live across tile iterations
// spills the codelet registers at every block size, so the loop-free form is
// used.)
template <int CBT>
__global__ void __launch_bounds__(CBT, 1024 / CBT) k_batch(const TileDesc *__restrict__ q, int ntiles, int ahead) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *s = reinterpret_cast<float2 *>(smem_raw);
    __shared__ TileDesc sd, sn;  // descriptor fields are re-read from shared memory, not held in registers
    const int t = blockIdx.x;
    if (t >= ntiles) return;
    const int tn = t + ahead;  // the tile that takes this slot a wave later
    if (threadIdx.x == 0) {
        sd = q[t];
        if (ahead > 0 && tn < ntiles) sn = q[tn];
    }
    __syncthreads();
    if (ahead > 0 && tn < ntiles) prefetch_tile(sn, threadIdx.x, blockDim.x);
    batch_tile(sd, s);
}

// Columns of long transforms (one column fills a CTA): a 4-CTA cluster takes
// up to 4 adjacent columns, one column per CTA.  CTA c reads rows
// [c*Q, (c+1)*Q) of all the columns with the column index fastest -- every
// matrix row is one contiguous segment -- and stores each value into the
// owning CTA's shared memory (distributed shared memory, natural order); after
// a cluster barrier every CTA runs its column's passes locally (the first pass
// reads the natural order, the last writes the padded rows); after a second
// barrier CTA c writes rows [c*Q, (c+1)*Q) of all the columns, read from the
// owners' shared memory, and a third barrier keeps every CTA's shared memory
// alive until the others have read it.  Every thread of the cluster reaches
// every barrier: CTAs without a column skip only the passes.
constexpr int kColCluster = 4;

__device__ __forceinline__ void col_passes(float2 *s, int ld, unsigned long long packed, const float2 *twg,
                                           const uint4 *pc) {
    int fi = 0;
    while (fi < kRadices - 1 && pass_count(packed, fi) == 0) fi++;
    const uint4 pc0 = __ldg(&pc[0]);
    int Rf = 2;
#define JV_DENSE_FIRST(R) (smem_pass<float, R, BEMAX, 1>(s, ld, 1, 1, twg, pc0), Rf = R)
    JV_RADIX_SWITCH(fi, JV_DENSE_FIRST)
#undef JV_DENSE_FIRST
    int Ns = Rf, p = 1;
    const float2 *tp = twg + Rf;
    smem_passes_from<float, BEMAX>(s, ld, 1, packed - (1ull << (4 * fi)), tp, pc, Ns, p);
}

__global__ void __cluster_dims__(kColCluster, 1, 1) __launch_bounds__(BT, 1)
    k_batch_cols(const TileDesc *__restrict__ q, int ntiles) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *s = reinterpret_cast<float2 *>(smem_raw);
    __shared__ TileDesc sd;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int t = blockIdx.x / kColCluster;  // the same descriptor for the whole cluster
    if (t >= ntiles) return;                 // uniform over the cluster
    if (threadIdx.x == 0) sd = q[t];
    __syncthreads();
    // each phase reads its values from the shared descriptor, so none of them
    // stays live in registers across the passes (which use all 64)
    {
        // ---- load: (row, column) with the column fastest, four loads in flight
        const int tid = threadIdx.x, nthr = blockDim.x;
        const int N = sd.N, nt = sd.nt;
        const int Q = (N + kColCluster - 1) / kColCluster;
        const int n0 = rank * Q, nr = max(0, min(N, n0 + Q) - n0);
        const int tot = nr * nt;
        const unsigned mnt = sd.mnt;
        const float2 *in = reinterpret_cast<const float2 *>(sd.in) + (sd.in_off + sd.v0 * sd.in_vs);
        const long ies = sd.in_es, ivs = sd.in_vs;
        const float sgn = sd.inv ? -1.f : 1.f;
        for (int i0 = tid; i0 < tot; i0 += 4 * nthr) {
            float2 c[4];
            int kk[4], nn[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int i = i0 + u * nthr;
                kk[u] = 0;
                nn[u] = 0;
                if (i < tot) {
                    const int r = mdiv(i, mnt);
                    kk[u] = i - r * nt;
                    nn[u] = n0 + r;
                    c[u] = in[(long)kk[u] * ivs + (long)nn[u] * ies];
                }
            }
#pragma unroll
            for (int u = 0; u < 4; u++) {
                if (i0 + u * nthr < tot) {
                    float2 *dst = cl.map_shared_rank(s, kk[u]);
                    dst[nn[u]] = make_float2(c[u].x, c[u].y * sgn);
                }
            }
        }
    }
    cl.sync();
    if ((int)cl.block_rank() < sd.nt) col_passes(s, sd.ld, sd.passes, sd.twg, sd.pc);
    cl.sync();
    {
        // ---- store: rows [n0, n0 + nr) of the columns, from their owners
        const int tid = threadIdx.x, nthr = blockDim.x;
        const int N = sd.N, nt = sd.nt;
        const int Q = (N + kColCluster - 1) / kColCluster;
        const int n0 = (int)cl.block_rank() * Q, nr = max(0, min(N, n0 + Q) - n0);
        const int tot = nr * nt;
        const unsigned mnt = sd.mnt;
        float2 *out = reinterpret_cast<float2 *>(sd.out) + (sd.out_off + sd.v0 * sd.out_vs);
        const long oes = sd.out_es, ovs = sd.out_vs;
        const float scale = sd.has_scale ? sd.scale : 1.f, sy = (sd.inv ? -1.f : 1.f) * scale;
        for (int i = tid; i < tot; i += nthr) {
            const int r = mdiv(i, mnt), k = i - r * nt, n = n0 + r;
            const float2 *src = cl.map_shared_rank(s, k);
            const float2 v = src[spad(n)];
            out[(long)k * ovs + (long)n * oes] = make_float2(v.x * scale, v.y * sy);
        }
    }
    cl.sync();
}

// ---------------------------------------------------------------- host side
// A call the batch runs through the plain path instead of tiles: single-
// precision c2c columns (adjacent vectors on both sides) of 8192 points or
// more, which the plain calls take as two steps (on the register-resident
// column tiles or the shared-memory kernel, the groups along the grid's y).
// Measured on the 2 GB batch: its columns of 8192-16384 points 1.052 ms this
// way against 1.185 ms on the column clusters; columns of 3000-8191 points
// were slower this way than as tiles (0.94 against 0.72 ms).
struct StepCall {
    Plan *p;
    const vsip_cmview_f *x, *y;
};

struct BatchBuild {
    std::vector<TileDesc> tiles[kClasses];
    size_t smem[kClasses] = {0, 0, 0, 0};
    std::vector<StepCall> steps;
    double bytes = 0;
};

static long tile_ld(long N, bool vf) {
    long ld = (N - 1) + (N - 1) / 16 + 1;
    if (vf && (ld % 2 == 0)) ld += 1;
    return ld;
}

// FFTs per tile for length N (transforms adjacent in memory or not).
long batch_fft_per_tile(long N, bool vf, long rows);

static bool build_tiles(size_t n, const vsip_fftm_f *const plans[], const vsip_cmview_f *const in[],
                        const vsip_cmview_f *const out[], BatchBuild &bb) {
    Device *d = device();
    if (!d) return false;
    for (size_t i = 0; i < n; i++) {
        Plan *p = plan_of(plans[i]);
        if (!p || p->prec != P_F32 || (p->type != JV_CCFFTOP && p->type != JV_CCFFTIP)) {
            set_error(E_ARG, "batch: every plan must be a single-precision c2c plan");
            return false;
        }
        if (!p->smooth || !p->d_twg || !p->d_pc || p->radix.empty() || p->MN > BEMAX * BT) {
            set_error(E_UNSUPPORTED, "batch: lengths must be 2^a 3^b 5^c 7^d and at most 16384");
            return false;
        }
        const vsip_cmview_f *x = in[i];
        const vsip_cmview_f *y = (p->type == JV_CCFFTIP || !out || !out[i]) ? x : out[i];
        if (!x || !y || !x->block || !y->block) {
            set_error(E_ARG, "batch: null view");
            return false;
        }
        Mirror *mx = mirror_find(x->block), *my = mirror_find(y->block);
        if (!mx || !my || x->block->cstride != 2 || y->block->cstride != 2) {
            set_error(E_ARG, "batch: views must be of admitted interleaved blocks");
            return false;
        }
        const long N = p->MN, nv = p->mN;
        long xl = (long)(p->major == 0 ? x->row_length : x->col_length);
        long xn = (long)(p->major == 0 ? x->col_length : x->row_length);
        long yl = (long)(p->major == 0 ? y->row_length : y->col_length);
        long yn = (long)(p->major == 0 ? y->col_length : y->row_length);
        if (xl < N || xn < nv || yl < N || yn < nv) {
            set_error(E_ARG, "batch: view smaller than its plan");
            return false;
        }
        TileDesc t;
        memset(&t, 0, sizeof(t));
        t.in = (const float *)mx->d;
        t.out = (float *)my->d;
        t.in_off = (long)x->offset;
        t.out_off = (long)y->offset;
        if (p->major == 0) {
            t.in_es = x->row_stride;
            t.in_vs = x->col_stride;
            t.out_es = y->row_stride;
            t.out_vs = y->col_stride;
        } else {
            t.in_es = x->col_stride;
            t.in_vs = x->row_stride;
            t.out_es = y->col_stride;
            t.out_vs = y->row_stride;
        }
        // bounds of both views inside their blocks
        auto span_ok = [&](long off, long es, long vs, long len, long cnt, long size) {
            long lo = off + std::min(0L, (cnt - 1) * vs) + std::min(0L, (len - 1) * es);
            long hi = off + std::max(0L, (cnt - 1) * vs) + std::max(0L, (len - 1) * es);
            return lo >= 0 && hi < size;
        };
        if (!span_ok(t.in_off, t.in_es, t.in_vs, N, nv, (long)x->block->size) ||
            !span_ok(t.out_off, t.out_es, t.out_vs, N, nv, (long)y->block->size)) {
            set_error(E_ARG, "batch: view outside its block");
            return false;
        }
        if (x->block == y->block && (t.in_off != t.out_off || t.in_es != t.out_es || t.in_vs != t.out_vs)) {
            set_error(E_UNSUPPORTED, "batch: x and y on one block must be the same view");
            return false;
        }
        t.twg = (const float2 *)p->d_twg;
        t.pc = (const uint4 *)p->d_pc;
        t.N = (int)N;
        if (!pack_passes(p->radix, &t.passes)) {
            set_error(E_UNSUPPORTED, "batch: pass schedule outside the codelets");
            return false;
        }
        t.inv = (p->dir == 1) ? 1 : 0;
        t.has_scale = (p->scale != 1.0) ? 1 : 0;
        t.scale = (float)p->scale;
        bool vf_in = labs(t.in_vs) == 1 && labs(t.in_es) != 1;
        bool vf_out = labs(t.out_vs) == 1 && labs(t.out_es) != 1;
        t.vec_fast = (vf_in || vf_out) ? 1 : 0;
        t.ld = (int)tile_ld(N, t.vec_fast);
        if (N >= kLongFewMin && resident_long_columns_f(p, x, y)) {
            bb.steps.push_back(StepCall{p, x, y});
            bb.bytes += 16.0 * N * nv;
            continue;
        }
        if (t.vec_fast && 2 * N > BEMAX * BT) {
            // columns of long transforms: groups of up to kColCluster adjacent
            // columns, one cluster each (k_batch_cols)
            t.ld = (int)tile_ld(N, false);
            for (long v0 = 0; v0 < nv; v0 += kColCluster) {
                TileDesc u = t;
                u.v0 = v0;
                u.nt = (int)std::min((long)kColCluster, nv - v0);
                u.mnt = magic_host((unsigned long)u.nt);
                u.cls = (unsigned char)kColClass;
                bb.tiles[kColClass].push_back(u);
                bb.smem[kColClass] = std::max(bb.smem[kColClass], (size_t)u.ld * 8);
            }
            bb.bytes += 16.0 * N * nv;
            continue;
        }
        long per = batch_fft_per_tile(N, t.vec_fast, nv);
        // every pass of the tile must fit the CTA: a thread holds
        // pass_k(BEMAX, R) butterflies of radix R (the plan's schedule fits
        // one transform by construction)
        long min_pts = BEMAX;
        for (int r : p->radix) min_pts = std::min(min_pts, (long)r * pass_k(BEMAX, r));
        while (per > 1 && per * N > (long)BT * min_pts) per--;
        while (per > 1 && per * (long)t.ld * 8 > (long)d->smem_optin - 512) per--;
        for (long v0 = 0; v0 < nv; v0 += per) {
            TileDesc u = t;
            u.v0 = v0;
            u.nt = (int)std::min(per, nv - v0);
            u.mnt = magic_host((unsigned long)u.nt);
            // threads the tile's passes need: a thread holds pass_k(BEMAX, R) butterflies
            long need = 32;
            for (int r : p->radix) {
                const long K = pass_k(BEMAX, r);
                need = std::max(need, ((long)u.nt * N / r + K - 1) / K);
            }
            int c = 0;
            while (c < kClasses - 1 && need > kClassBT[c]) c++;
            u.cls = (unsigned char)c;
            bb.tiles[c].push_back(u);
            bb.smem[c] = std::max(bb.smem[c], (size_t)u.nt * u.ld * 8);
        }
        bb.bytes += 16.0 * N * nv;
    }
    // largest tiles first: each queue's tail is made of short work
    for (int c = 0; c < kClasses; c++)
        std::stable_sort(bb.tiles[c].begin(), bb.tiles[c].end(), [](const TileDesc &a, const TileDesc &b) {
            return (long)a.N * a.nt > (long)b.N * b.nt;
        });
    return true;
}

struct DevBatch {
    TileDesc *q = nullptr;            // the classes' queues, one after the other
    int off[kClasses] = {0, 0, 0, 0};  // first descriptor of each class
    int n[kClasses] = {0, 0, 0, 0};    // descriptors of each class
    size_t smem[kClasses] = {0, 0, 0, 0};
    int total = 0;
    std::vector<StepCall> steps;      // calls run through the plain path
};

static bool upload(const BatchBuild &bb, DevBatch &db) {
    // the step calls' plans get their scratch now (nothing may allocate while
    // a batch is recorded into its graph)
    db.steps = bb.steps;
    for (const StepCall &c : db.steps)
        if (!enqueue_resident_c2c_f(c.p, c.x, c.y, nullptr, true)) return false;
    std::vector<TileDesc> all;
    for (int c = 0; c < kClasses; c++) {
        db.off[c] = (int)all.size();
        db.n[c] = (int)bb.tiles[c].size();
        db.smem[c] = bb.smem[c];
        all.insert(all.end(), bb.tiles[c].begin(), bb.tiles[c].end());
    }
    db.total = (int)all.size();
    db.q = (TileDesc *)dmalloc(std::max<size_t>(1, all.size()) * sizeof(TileDesc));
    if (!db.q) return false;
    Device *d = device();
    if (!all.empty() && !cuda_ok(cudaMemcpyAsync(db.q, all.data(), all.size() * sizeof(TileDesc),
                                                 cudaMemcpyHostToDevice, d->stream),
                                 "batch queue upload"))
        return false;
    return true;
}

template <int CBT>
static bool launch_class(const DevBatch &db, int c, cudaStream_t st) {
    Device *d = device();
    static std::atomic<bool> attr{false};  // set once; concurrent first calls both set it
    if (!attr) {
        if (!cuda_ok(cudaFuncSetAttribute(k_batch<CBT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)d->smem_optin - 512),
                     "cudaFuncSetAttribute"))
            return false;
        attr = true;
    }
    // CTAs resident at once for this class: the descriptor that many places
    // further down the queue is the one a finishing CTA's slot takes next
    int per_sm = 0;
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<CBT>, CBT, db.smem[c]),
                 "batch occupancy"))
        return false;
    const int ahead = std::max(1, per_sm) * d->sms;
    k_batch<CBT><<<db.n[c], CBT, db.smem[c], st>>>(db.q + db.off[c], db.n[c], ahead);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_batch launch");
}

static bool launch_cols(const DevBatch &db, cudaStream_t st) {
    Device *d = device();
    static std::atomic<bool> attr{false};  // set once; concurrent first calls both set it
    if (!attr) {
        if (!cuda_ok(cudaFuncSetAttribute(k_batch_cols, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)d->smem_optin - 512),
                     "cudaFuncSetAttribute"))
            return false;
        attr = true;
    }
    const int c = kColClass;
    k_batch_cols<<<db.n[c] * kColCluster, BT, db.smem[c], st>>>(db.q + db.off[c], db.n[c]);
    count_launch();
    return cuda_ok(cudaGetLastError(), "k_batch_cols launch");
}

static bool launch_one(const DevBatch &db, int c, cudaStream_t st) {
    switch (c) {
        case 0: return launch_class<256>(db, c, st);
        case 1: return launch_class<512>(db, c, st);
        case 2: return launch_class<1024>(db, c, st);
        default: return launch_cols(db, st);
    }
}

// Streams and events the classes run on side by side (forked from and joined
// back to the caller's stream; the same pattern is recorded into the graph).
constexpr int kStepStreams = 4;  // streams of the calls run through the plain path
struct BatchStreams {
    cudaStream_t s[kClasses + kStepStreams] = {};  // the classes', then the plain-path calls'
    cudaEvent_t fork = nullptr, join[kClasses + kStepStreams] = {};
    bool ready = false;
};
static BatchStreams g_bs;
static std::mutex g_bs_mu;

static bool batch_streams() {
    std::lock_guard<std::mutex> lk(g_bs_mu);
    if (g_bs.ready) return true;
    bool ok = cuda_ok(cudaEventCreateWithFlags(&g_bs.fork, cudaEventDisableTiming), "batch event");
    for (int c = 0; c < kClasses + kStepStreams && ok; c++)
        ok = cuda_ok(cudaStreamCreateWithFlags(&g_bs.s[c], cudaStreamNonBlocking), "batch stream") &&
             cuda_ok(cudaEventCreateWithFlags(&g_bs.join[c], cudaEventDisableTiming), "batch event");
    g_bs.ready = ok;
    return ok;
}

// the plain-path calls on their streams; calls of one plan share its scratch,
// so they all go to one stream, in order
static int step_stream(const StepCall &c) { return (int)(((uintptr_t)c.p >> 6) % kStepStreams); }

static bool launch(const DevBatch &db, cudaStream_t st) {
    if (db.total == 0 && db.steps.empty()) return true;
    int used = 0, only = 0;
    for (int c = 0; c < kClasses; c++)
        if (db.n[c]) {
            used++;
            only = c;
        }
    if (used == 1 && db.steps.empty()) return launch_one(db, only, st);
    if (!batch_streams()) return false;
    bool ok = cuda_ok(cudaEventRecord(g_bs.fork, st), "batch fork");
    if (!db.steps.empty()) {
        bool on[kStepStreams] = {};
        for (const StepCall &c : db.steps) {
            const int k = step_stream(c);
            cudaStream_t sl = g_bs.s[kClasses + k];
            if (!on[k]) ok = ok && cuda_ok(cudaStreamWaitEvent(sl, g_bs.fork, 0), "batch fork");
            on[k] = true;
            ok = ok && enqueue_resident_c2c_f(c.p, c.x, c.y, sl, false);
        }
        for (int k = 0; k < kStepStreams && ok; k++)
            if (on[k])
                ok = cuda_ok(cudaEventRecord(g_bs.join[kClasses + k], g_bs.s[kClasses + k]), "batch join") &&
                     cuda_ok(cudaStreamWaitEvent(st, g_bs.join[kClasses + k], 0), "batch join");
    }
    // largest CTAs first: they hold the longest tiles
    for (int c = kClasses - 1; c >= 0 && ok; c--) {
        if (!db.n[c]) continue;
        ok = cuda_ok(cudaStreamWaitEvent(g_bs.s[c], g_bs.fork, 0), "batch fork") && launch_one(db, c, g_bs.s[c]) &&
             cuda_ok(cudaEventRecord(g_bs.join[c], g_bs.s[c]), "batch join") &&
             cuda_ok(cudaStreamWaitEvent(st, g_bs.join[c], 0), "batch join");
    }
    return ok;
}

static void free_dev(DevBatch &db) {
    dfree(db.q);
    db.q = nullptr;
}

}  // namespace jv

using namespace jv;

struct jvsip_fftm_batchplan_s {
    DevBatch db;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const void *> blocks;  // output blocks, marked device-newer after a run
};

static void mark_outputs(size_t n, const vsip_fftm_f *const plans[], const vsip_cmview_f *const in[],
                         const vsip_cmview_f *const out[]) {
    for (size_t i = 0; i < n; i++) {
        Plan *p = plan_of(plans[i]);
        const vsip_cmview_f *y = (p->type == JV_CCFFTIP || !out || !out[i]) ? in[i] : out[i];
        Mirror *m = mirror_find(y->block);
        if (m) m->device_newer = true;
    }
}

extern "C" {

int jvsip_fftm_batch_f(size_t n, const vsip_fftm_f *const plans[], const vsip_cmview_f *const in[],
                       const vsip_cmview_f *const out[]) {
    if (n == 0) return 0;
    if (!plans || !in) {
        set_error(E_ARG, "batch: null arrays");
        return E_ARG;
    }
    BatchBuild bb;
    if (!build_tiles(n, plans, in, out, bb)) return jvsip_gpu_last_error();
    DevBatch db;
    Device *d = device();
    bool ok = upload(bb, db) && launch(db, d->stream);
    free_dev(db);  // stream-ordered reuse of the pool
    if (!ok) return jvsip_gpu_last_error() ? jvsip_gpu_last_error() : E_CUDA;
    mark_outputs(n, plans, in, out);
    return 0;
}

jvsip_fftm_batchplan_f *jvsip_fftm_batch_create_f(size_t n, const vsip_fftm_f *const plans[],
                                                  const vsip_cmview_f *const in[], const vsip_cmview_f *const out[]) {
    if (!plans || !in) {
        set_error(E_ARG, "batch: null arrays");
        return nullptr;
    }
    BatchBuild bb;
    if (!build_tiles(n, plans, in, out, bb)) return nullptr;
    jvsip_fftm_batchplan_f *b = new (std::nothrow) jvsip_fftm_batchplan_f();
    if (!b) {
        set_error(E_ALLOC, "batch plan");
        return nullptr;
    }
    Device *d = device();
    if (!upload(bb, b->db) || !cuda_ok(cudaStreamSynchronize(d->stream), "batch upload")) {
        free_dev(b->db);
        delete b;
        return nullptr;
    }
    // record the launch once; runs replay the graph
    cudaStream_t cs = nullptr;
    bool ok = cuda_ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream");
    ok = ok && cuda_ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (ok) {
        bool lk = launch(b->db, cs);
        ok = cuda_ok(cudaStreamEndCapture(cs, &b->graph), "end capture") && lk;
    }
    ok = ok && cuda_ok(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    if (cs) cudaStreamDestroy(cs);
    if (!ok) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        free_dev(b->db);
        delete b;
        return nullptr;
    }
    for (size_t i = 0; i < n; i++) {
        Plan *p = plan_of(plans[i]);
        const vsip_cmview_f *y = (p->type == JV_CCFFTIP || !out || !out[i]) ? in[i] : out[i];
        b->blocks.push_back(y->block);
    }
    return b;
}

int jvsip_fftm_batch_run_f(jvsip_fftm_batchplan_f *b) {
    if (!b) return E_ARG;
    Device *d = device();
    if (!d) return E_NODEVICE;
    if (b->db.total == 0 && b->db.steps.empty()) return 0;
    if (!cuda_ok(cudaGraphLaunch(b->exec, d->stream), "batch graph launch")) return E_CUDA;
    count_launch();
    for (const void *blk : b->blocks) {
        Mirror *m = mirror_find(blk);
        if (m) m->device_newer = true;
    }
    return 0;
}

int jvsip_fftm_loop_f(size_t n, const vsip_fftm_f *const plans[], const vsip_cmview_f *const in[],
                      const vsip_cmview_f *const out[]) {
    if (n && (!plans || !in)) {
        set_error(E_ARG, "loop: null arrays");
        return E_ARG;
    }
    for (size_t i = 0; i < n; i++) {
        Plan *p = plan_of(plans[i]);
        if (!p) {
            set_error(E_ARG, "loop: not a plan of this library");
            return E_ARG;
        }
        if (p->type == JV_CCFFTIP || !out || !out[i]) vsip_ccfftmip_f(plans[i], in[i]);
        else vsip_ccfftmop_f(plans[i], in[i], out[i]);
        const int e = jvsip_gpu_last_error();
        if (e) return e;
    }
    return 0;
}

int jvsip_fftm_batch_destroy_f(jvsip_fftm_batchplan_f *b) {
    if (!b) return 0;
    Device *d = device();
    if (d) cudaStreamSynchronize(d->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    free_dev(b->db);
    delete b;
    return 0;
}

}  // extern "C"
