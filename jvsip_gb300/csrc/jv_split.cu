// jv_split.cu -- precision form: 1024-point rows as two tensor-core DFT
// products with hi/lo-split 16-bit operands and FP32 accumulation.
//
// A row x (n = 32a + b) is a 32 x 32 matrix X[a][b].  Its DFT is the
// four-step  Z = F32^T-applied over a,  Z'[c][b] = Z[c][b] * w1024^(bc),
// X[c + 32d] = sum_b Z'[c][b] w32^(bd).  Each step is a real GEMM whose A
// operand is 128 x 128 (4 rows x 32 vectors; K = {hi, lo} x {re, im} x 32)
// and whose B operand is 64 x 128 (the 32-point DFT matrix in the 2x2 real
// form of complex multiplication, K = {W_hi, W_lo} x {re, im} x 32).  Three
// products accumulate into one FP32 tensor-memory tile:
//     X_hi * W_hi  +  X_lo * W_hi  +  X_hi * W_lo
// (A K-blocks 0-3 with B 0-3, A 4-7 with B 0-3, A 0-3 with B 4-7), which
// recovers about 22 (FP16) or 16 (BF16) significant bits of each operand.
// FP16 operands are scaled per row by a power of two before the split (so
// their range fits FP16); BF16 operands are not scaled.  The inverse
// direction runs as conj(F(conj x)); the user scale is applied at the store.
//
// Per CTA: 128 threads, one warp per row; 64 tensor-memory columns hold the
// 128 x 64 FP32 accumulator of step 1 and then of step 2; one elected thread
// issues 12 tcgen05.mma per step and commits them to an mbarrier the CTA
// waits on with a bounded loop.  The A operand's K-blocks are 2064 bytes
// apart (2048 + 16) so that the step-2 stores, which run along K, spread
// over all shared-memory banks.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <string.h>

#include <math.h>
#include <stdlib.h>

#include <mutex>
#include <vector>

#include "jv_core.h"
#include "jv_tc.cuh"

namespace jv {

constexpr int SPN = 1024;                        // transform length of the form
constexpr int SPM = 128;                         // GEMM M: 4 rows x 32
constexpr int SPK = 128;                         // operand K: {hi, lo} x {re, im} x 32
constexpr int SPNN = 64;                         // GEMM N: {re, im} x 32
constexpr uint32_t SP_A_LBO = (SPM / 8) * 128 + 16;  // bytes between K-adjacent core matrices of A
constexpr uint32_t SP_B_LBO = (SPNN / 8) * 128;      // the same for B (unpadded)
constexpr int SP_A_BYTES = (SPK / 8) * SP_A_LBO;     // 33024
constexpr int SP_B_BYTES = (SPK / 8) * SP_B_LBO;     // 16384
constexpr int SP_TMEM_COLS = 64;
constexpr uint32_t SP_WAIT_LIMIT = 1u << 24;

// byte offset of element (row, k) of a K-major no-swizzle operand made of
// 8-row x 16-byte core matrices: [k/8] (lbo apart) [row/8] (128 apart) [row%8][k%8]
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, uint32_t lbo) {
    return (uint32_t)(k >> 3) * lbo + (uint32_t)((row >> 3) << 7) + (uint32_t)((row & 7) << 4) + (uint32_t)((k & 7) << 1);
}

struct SplitArgs {
    const float2 *in;
    float2 *out;
    long off_in, vs_in, off_out, vs_out;
    long nvec;
    int inv, has_scale;
    float scale;
    const uint4 *bop;     // B operand, SP_B_BYTES in core-matrix layout
    const float2 *tw;     // [c][b] = exp(-2 pi i bc/1024), c, b < 32
    int *status;          // set to 1 when a barrier wait expired
    int bulk_rows;        // input rows start on 16-byte boundaries: loaded by bulk copies
    int bulk_out;         // output rows start on 16-byte boundaries: stored by bulk copies
};

// two floats -> one 32-bit word of two 16-bit values (first in the low half),
// and back
template <bool BF>
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    uint32_t u;
    if (BF) {
        __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
        memcpy(&u, &h, 4);
    } else {
        __half2 h = __floats2half2_rn(lo, hi);
        memcpy(&u, &h, 4);
    }
    return u;
}
template <bool BF>
__device__ __forceinline__ float2 unpack2(uint32_t u) {
    if (BF) {
        __nv_bfloat162 h;
        memcpy(&h, &u, 4);
        return __bfloat1622float2(h);
    }
    __half2 h;
    memcpy(&h, &u, 4);
    return __half22float2(h);
}
// hi word and lo word of the split of (x0, x1)
template <bool BF>
__device__ __forceinline__ void split2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
    hi = pack2<BF>(x0, x1);
    const float2 f = unpack2<BF>(hi);
    lo = pack2<BF>(x0 - f.x, x1 - f.y);
}

// power-of-two scale bringing the warp's largest magnitude into [2^13, 2^14)
__device__ __forceinline__ float warp_scale(float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (!(m > 0.f) || !isfinite(m)) return 1.f;
    int e = ilogbf(m);
    return ldexpf(1.f, 13 - e);
}

// the three products of one step into tensor memory at `d`
__device__ __forceinline__ void split_mma(uint32_t d, uint32_t a0, uint32_t b0, uint32_t idesc) {
#pragma unroll 1
    for (int i = 0; i < 12; i++) {
        const int ka = (i < 8) ? i : i - 8;  // A K-chunk: hi 0-3, lo 4-7, hi 0-3
        const int kb = (i < 4) ? i : i - 4;  // B K-chunk: W_hi 0-3, W_hi 0-3, W_lo 4-7
        tc::mma_f16(d, tc::smem_desc(a0 + ka * 2 * SP_A_LBO, SP_A_LBO, 128),
                    tc::smem_desc(b0 + kb * 2 * SP_B_LBO, SP_B_LBO, 128), idesc, i > 0);
    }
}

// 32 accumulator columns of this warp's lanes, from column `col`
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    float t[16];
    tc::tmem_ld16(taddr, t);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = t[i];
    tc::tmem_ld16(taddr + 16, t);
#pragma unroll
    for (int i = 0; i < 16; i++) v[16 + i] = t[i];
}

// ---- the steps of one group of 4 rows, shared by both kernels

// step 1 operand from the thread's vector b = l of row w (v[a] = x[32a + l],
// scaled by s1): A1[(w, b)][part*64 + ri*32 + a], K-blocks ab (re hi), 4+ab
// (im hi), 8+ab (re lo), 12+ab (im lo)
template <bool BF>
__device__ __forceinline__ void sp_operand1(unsigned char *Asm, int w, int l, const float2 (&v)[32], float s1) {
    unsigned char *arow = Asm + core_off(w * 32 + l, 0, SP_A_LBO);
#pragma unroll
    for (int ab = 0; ab < 4; ab++) {
        uint4 hr, hi, lr, li;
        uint32_t *phr = &hr.x, *phi = &hi.x, *plr = &lr.x, *pli = &li.x;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 e0 = v[ab * 8 + 2 * q], e1 = v[ab * 8 + 2 * q + 1];
            split2<BF>(e0.x * s1, e1.x * s1, phr[q], plr[q]);
            split2<BF>(e0.y * s1, e1.y * s1, phi[q], pli[q]);
        }
        *reinterpret_cast<uint4 *>(arow + (0 + ab) * SP_A_LBO) = hr;
        *reinterpret_cast<uint4 *>(arow + (4 + ab) * SP_A_LBO) = hi;
        *reinterpret_cast<uint4 *>(arow + (8 + ab) * SP_A_LBO) = lr;
        *reinterpret_cast<uint4 *>(arow + (12 + ab) * SP_A_LBO) = li;
    }
}

// step 1 result (lane (w, l) = (row, b), columns re c | im c) times the
// twiddle w1024^(b c), then the step 2 operand A2[(w, c)][part*64 + ri*32 + b]
// written over step 1's; returns the step's power-of-two scale.  Lane pairs
// (l, l^1) trade one word so that each lane stores two 4-byte pairs of
// adjacent b: even lanes (re hi, im hi) at b = l, odd lanes (re lo, im lo) at
// b = l - 1; the two stores are ordered so the even and odd halves of the
// warp fall in different banks.
template <bool BF>
__device__ __forceinline__ float sp_operand2(unsigned char *Asm, int w, int l, float (&zr)[32], float (&zi)[32],
                                             const float2 *__restrict__ tw) {
    float mx = 0.f;
#pragma unroll
    for (int c = 0; c < 32; c++) {
        const float2 t = __ldg(&tw[c * 32 + l]);
        const float r = zr[c] * t.x - zi[c] * t.y, i = zr[c] * t.y + zi[c] * t.x;
        zr[c] = r;
        zi[c] = i;
        mx = fmaxf(mx, fmaxf(fabsf(r), fabsf(i)));
    }
    const float s2 = BF ? 1.f : warp_scale(mx);
    const bool even = (l & 1) == 0;
    const int k1 = even ? l : 96 + l - 1, k2 = even ? 32 + l : 64 + l - 1;
    unsigned char *p1 = Asm + core_off(w * 32, k1, SP_A_LBO);
    unsigned char *p2 = Asm + core_off(w * 32, k2, SP_A_LBO);
#pragma unroll
    for (int c = 0; c < 32; c++) {
        uint32_t P, Q;  // (re hi | im hi << 16), (re lo | im lo << 16)
        split2<BF>(zr[c] * s2, zi[c] * s2, P, Q);
        const uint32_t R = __shfl_xor_sync(0xffffffffu, even ? Q : P, 1);
        const uint32_t X = even ? P : R, Y = even ? R : Q;
        const uint32_t wlo = __byte_perm(X, Y, 0x5410), whi = __byte_perm(X, Y, 0x7632);
        const uint32_t mo = (uint32_t)((c >> 3) << 7) + (uint32_t)((c & 7) << 4);
        *reinterpret_cast<uint32_t *>(p1 + mo) = even ? wlo : whi;
        *reinterpret_cast<uint32_t *>(p2 + mo) = even ? whi : wlo;
    }
    return s2;
}

// step 2 result: lane (w, l) = (row, c = l), columns re d | im d -> out[c + 32 d]
// With output rows on 16-byte boundaries the rows are staged in the A
// operand's space (free once step 2's MMAs completed) and written by one bulk
// copy each, issued by thread 0, which waits until the copies have read the
// stage (the CTA's shared memory outlives them).
__device__ __forceinline__ void sp_store(const SplitArgs &a, uint32_t lane_base, long row, int l, float f,
                                         unsigned char *Asm, int tid) {
    float yr[32], yi[32];
    tmem_ld32(lane_base + 0, yr);
    tmem_ld32(lane_base + 32, yi);
    tc::tmem_ld_wait();
    if (a.bulk_out) {
        const int w = tid >> 5;
        float2 *stg = reinterpret_cast<float2 *>(Asm) + w * SPN;
#pragma unroll
        for (int d = 0; d < 32; d++) {
            float2 o = make_float2(yr[d] * f, yi[d] * f);
            if (a.inv) o.y = -o.y;
            stg[l + 32 * d] = o;
        }
        tc::fence_async_smem();
        __syncthreads();
        if (tid == 0) {
            const long row0 = row - w;
            const int nr = (int)min(4L, a.nvec - row0);
            for (int r = 0; r < nr; r++)
                tc::bulk_store(a.out + a.off_out + (row0 + r) * a.vs_out, Asm + r * SPN * 8, SPN * 8);
            tc::bulk_commit();
            tc::bulk_wait_read();
        }
        return;
    }
    if (row < a.nvec) {
        float2 *dst = a.out + a.off_out + row * a.vs_out;
#pragma unroll
        for (int d = 0; d < 32; d++) {
            float2 o = make_float2(yr[d] * f, yi[d] * f);
            if (a.inv) o.y = -o.y;
            dst[l + 32 * d] = o;
        }
    }
}

// Steps 1 and 2 of the group whose rows the threads hold in v (conjugated when
// inverse): operand, MMAs, twiddle, operand, MMAs, store.  Returns false when
// a barrier wait expired (uniform over the CTA); *pending is then the MMA
// barrier phase still outstanding (2: none).
template <bool BF>
__device__ __forceinline__ bool sp_group(const SplitArgs &a, unsigned char *Asm, uint32_t a0, uint32_t b0,
                                         uint32_t tbase, uint64_t *mbar, float2 (&v)[32], long row, int tid,
                                         uint32_t *pending) {
    const int w = tid >> 5, l = tid & 31;
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < 32; i++) mx = fmaxf(mx, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
    const float s1 = BF ? 1.f : warp_scale(mx);
    sp_operand1<BF>(Asm, w, l, v, s1);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t idesc = tc::idesc_f16(SPM, SPNN, BF ? 1 : 0);
    if (tid == 0) {
        split_mma(tbase, a0, b0, idesc);
        tc::mma_commit(mbar);
    }
    bool ok = tc::mbar_wait(mbar, 0, SP_WAIT_LIMIT);
    ok = __syncthreads_and(ok);
    *pending = ok ? 2u : 0u;
    tc::fence_after_sync();
    if (!ok) return false;
    const uint32_t lane_base = tbase + ((uint32_t)(w * 32) << 16);
    float zr[32], zi[32];
    tmem_ld32(lane_base + 0, zr);
    tmem_ld32(lane_base + 32, zi);
    tc::tmem_ld_wait();
    const float s2 = sp_operand2<BF>(Asm, w, l, zr, zi, a.tw);
    // the step 1 accumulator is read out: step 2 reuses its columns
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
        split_mma(tbase, a0, b0, idesc);
        tc::mma_commit(mbar);
    }
    ok = tc::mbar_wait(mbar, 1, SP_WAIT_LIMIT);
    ok = __syncthreads_and(ok);
    *pending = ok ? 2u : 1u;
    tc::fence_after_sync();
    if (!ok) return false;
    sp_store(a, lane_base, row, l, (a.has_scale ? a.scale : 1.f) / (s1 * s2), Asm, tid);
    // the accumulator is read out before the next group's step 1 writes it
    tc::fence_before_sync();
    return true;
}

// One group per CTA (any 8-byte aligned rows).
template <bool BF>
__global__ void __launch_bounds__(128, 4) k_split1024(const SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *Bsm = smem;                     // 16 KiB
    unsigned char *Asm = smem + SP_B_BYTES;        // 33024 bytes
    __shared__ __align__(8) uint64_t mbar, bbar, ibar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    const long row0 = (long)blockIdx.x * 4, row = row0 + w;
    const bool live = row < a.nvec;
    const int nr = (int)min(4L, a.nvec - row0);
    if (w == 0) {
        tc::tmem_alloc(&tslot, SP_TMEM_COLS);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        tc::mbar_init(&mbar, 1);
        // the B operand (constant per plan) by one bulk copy, and with rows on
        // 16-byte boundaries the group's rows by one bulk copy each into the A
        // operand's space (free until step 1's operand is written)
        tc::mbar_init(&bbar, 1);
        tc::mbar_expect_tx(&bbar, SP_B_BYTES);
        tc::bulk_load(Bsm, a.bop, SP_B_BYTES, &bbar);
        if (a.bulk_rows) {
            tc::mbar_init(&ibar, 1);
            tc::mbar_expect_tx(&ibar, (uint32_t)(nr * SPN * 8));
            for (int r = 0; r < nr; r++)
                tc::bulk_load(Asm + r * SPN * 8, a.in + a.off_in + (row0 + r) * a.vs_in, SPN * 8, &ibar);
        }
    }
    // thread (w, l) owns vector b = l of row w: x[32a + l], a < 32
    float2 v[32];
    bool ok = true;
    if (a.bulk_rows) {
        __syncthreads();  // the barrier is initialised
        ok = tc::mbar_wait(&ibar, 0, SP_WAIT_LIMIT);
        const float2 *src = reinterpret_cast<const float2 *>(Asm) + w * SPN;
#pragma unroll
        for (int i = 0; i < 32; i++) {
            float2 c = (live && ok) ? src[32 * i + l] : make_float2(0.f, 0.f);
            if (a.inv) c.y = -c.y;
            v[i] = c;
        }
    } else {
        const float2 *src = a.in + a.off_in + (live ? row : 0) * a.vs_in;
#pragma unroll
        for (int i = 0; i < 32; i++) {
            float2 c = live ? src[32 * i + l] : make_float2(0.f, 0.f);
            if (a.inv) c.y = -c.y;
            v[i] = c;
        }
    }
    tc::fence_before_sync();
    ok = __syncthreads_and(ok);  // also: every thread has read its row from the A space
    tc::fence_after_sync();
    uint32_t pending = 2u;
    if (!ok && a.bulk_rows) tc::mbar_wait(&ibar, 0, SP_WAIT_LIMIT);
    ok = ok && __syncthreads_and(tc::mbar_wait(&bbar, 0, SP_WAIT_LIMIT));
    if (ok) ok = sp_group<BF>(a, Asm, tc::smem_addr(Asm), tc::smem_addr(Bsm), tslot, &mbar, v, row, tid, &pending);
    else tc::mbar_wait(&bbar, 0, SP_WAIT_LIMIT);  // the copy ends before the CTA's shared memory is released
    if (!ok) {
        if (tid == 0) atomicExch(a.status, 1);
        // let MMAs still in flight finish (bounded) before the tensor memory is freed
        if (pending < 2u) tc::mbar_wait(&mbar, pending, SP_WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_dealloc(tslot, SP_TMEM_COLS);
}

// ---------------------------------------------------------------- host side
// B operand of both steps: row n = ro*32 + c, column k = part*64 + ri*32 + a,
// the real 2x2 form of w32^(ac) = exp(-2 pi i ac/32) (FP64, then split):
// (ro, ri) = (re, re): cos, (re, im): -sin, (im, re): +sin, (im, im): cos;
// part 0 holds the 16-bit rounding W_hi of each entry, part 1 the rounding
// W_lo of its remainder.
template <bool BF>
static std::vector<uint16_t> b_operand() {
    std::vector<uint16_t> b(SP_B_BYTES / 2, 0);
    const double pi = 3.14159265358979323846264338327950288;
    for (int ro = 0; ro < 2; ro++)
        for (int c = 0; c < 32; c++)
            for (int ri = 0; ri < 2; ri++)
                for (int aa = 0; aa < 32; aa++) {
                    double ang = -2.0 * pi * (double)((aa * c) % 32) / 32.0;
                    double wr = cos(ang), wi = sin(ang);
                    // Z = sum x w: re = xr wr - xi wi, im = xr wi + xi wr
                    double val = (ro == 0) ? (ri == 0 ? wr : -wi) : (ri == 0 ? wi : wr);
                    float vf = (float)val;
                    uint16_t hi, lo;
                    if (BF) {
                        __nv_bfloat16 h = __float2bfloat16_rn(vf);
                        hi = __bfloat16_as_ushort(h);
                        lo = __bfloat16_as_ushort(__float2bfloat16_rn((float)(val - (double)__bfloat162float(h))));
                    } else {
                        __half h = __float2half_rn(vf);
                        hi = __half_as_ushort(h);
                        lo = __half_as_ushort(__float2half_rn((float)(val - (double)__half2float(h))));
                    }
                    const int n = ro * 32 + c;
                    b[core_off(n, 0 * 64 + ri * 32 + aa, SP_B_LBO) / 2] = hi;
                    b[core_off(n, 1 * 64 + ri * 32 + aa, SP_B_LBO) / 2] = lo;
                }
    return b;
}

static std::mutex g_sp_mu;
static void *g_bop[2] = {nullptr, nullptr};
static void *g_tw = nullptr;
static int *g_status = nullptr;

static bool split_tables() {
    if (g_bop[0] && g_bop[1] && g_tw && g_status) return true;
    std::vector<uint16_t> b16 = b_operand<false>(), bbf = b_operand<true>();
    std::vector<float> w(2 * 32 * 32);
    for (int c = 0; c < 32; c++)
        for (int bb = 0; bb < 32; bb++) {
            double ang = -2.0 * 3.14159265358979323846264338327950288 * (double)(bb * c) / SPN;
            w[2 * (c * 32 + bb)] = (float)cos(ang);
            w[2 * (c * 32 + bb) + 1] = (float)sin(ang);
        }
    g_bop[0] = dmalloc(SP_B_BYTES);
    g_bop[1] = dmalloc(SP_B_BYTES);
    g_tw = dmalloc(w.size() * sizeof(float));
    g_status = (int *)dmalloc(sizeof(int));
    if (!g_bop[0] || !g_bop[1] || !g_tw || !g_status) return false;
    return cuda_ok(cudaMemcpy(g_bop[0], b16.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_bop[1], bbf.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_tw, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemset(g_status, 0, sizeof(int)), "split status");
}

// true when the split form ran (or failed with an error recorded); false when
// the call does not qualify and the plain kernels should run instead
bool launch_split_f32(const Job &j, cudaStream_t st) {
    if (j.form != JVSIP_FORM_SPLIT_BF16 && j.form != JVSIP_FORM_SPLIT_FP16) return false;
    if (j.kind != K_C2C || j.prec != P_F32 || j.N != SPN || j.nvec <= 0) return false;
    const CView &ci = j.cin, &co = j.cout;
    if (ci.cst != 2 || co.cst != 2 || ci.es != 1 || co.es != 1) return false;
    if ((const float *)ci.im != (const float *)ci.re + 1 || (const float *)co.im != (const float *)co.re + 1) return false;
    if (((uintptr_t)ci.re % 8) || ((uintptr_t)co.re % 8)) return false;
    if (labs(ci.vs) < SPN || labs(co.vs) < SPN) return false;
    {
        std::lock_guard<std::mutex> lk(g_sp_mu);
        if (!split_tables()) return true;
    }
    const bool bf = (j.form == JVSIP_FORM_SPLIT_BF16);
    SplitArgs a;
    a.in = (const float2 *)ci.re;
    a.out = (float2 *)co.re;
    a.off_in = ci.off;
    a.vs_in = ci.vs;
    a.off_out = co.off;
    a.vs_out = co.vs;
    a.nvec = j.nvec;
    a.inv = j.inv;
    a.has_scale = j.has_scale;
    a.scale = (float)j.scale;
    a.bop = (const uint4 *)g_bop[bf ? 1 : 0];
    a.tw = (const float2 *)g_tw;
    a.status = g_status;
    // operand reads: A chunks start at 2 * ka * SP_A_LBO (ka < 8) and span two
    // K-blocks of 16 x 128 bytes, ending at byte 16 * SP_A_LBO - 17 of A; B
    // chunks end at byte 16 * SP_B_LBO - 1 of B: both inside their operands
    const long ngroups = (j.nvec + 3) / 4;
    a.bulk_rows = ((uintptr_t)ci.re % 16) == 0 && (ci.off % 2) == 0 && (j.nvec == 1 || (ci.vs % 2) == 0);
    a.bulk_out = ((uintptr_t)co.re % 16) == 0 && (co.off % 2) == 0 && (j.nvec == 1 || (co.vs % 2) == 0);
    const size_t smem = SP_A_BYTES + SP_B_BYTES;
    static std::atomic<bool> attr[2]{};  // set once per form; concurrent first calls both set it
    if (!attr[bf]) {
        cudaError_t e = bf ? cudaFuncSetAttribute(k_split1024<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                           : cudaFuncSetAttribute(k_split1024<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!cuda_ok(e, "cudaFuncSetAttribute")) return true;
        attr[bf] = true;
    }
    if (bf) k_split1024<true><<<(unsigned)ngroups, 128, smem, st>>>(a);
    else k_split1024<false><<<(unsigned)ngroups, 128, smem, st>>>(a);
    count_launch();
    cuda_ok(cudaGetLastError(), "k_split1024 launch");
    return true;
}

// Device status of the split kernels (a bounded wait that gave up); read and
// cleared at synchronisation points.  Returns 0 when clean.
int split_status_check(cudaStream_t st) {
    std::lock_guard<std::mutex> lk(g_sp_mu);
    if (!g_status) return 0;
    int h = 0;
    if (cudaMemcpyAsync(&h, g_status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return E_CUDA;
    if (h) {
        cudaMemsetAsync(g_status, 0, sizeof(int), st);
        set_error(E_DEVICE, "tensor-core barrier wait expired in the split-precision kernel");
        return E_DEVICE;
    }
    return 0;
}

}  // namespace jv
