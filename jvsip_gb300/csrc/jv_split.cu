// jv_split.cu -- precision form: 1024-point rows as two tensor-core DFT
// products with hi/lo-split 16-bit operands and FP32 accumulation.
//
// A row x (n = 32a + b) is a 32 x 32 matrix X[a][b].  Its DFT is the
// four-step  Z[b][c] = sum_a X[a][b] w32^(ac),  Z'[b][c] = Z[b][c] w1024^(bc),
// X[c + 32d] = sum_b Z'[b][c] w32^(bd).  Each step is a real GEMM whose A
// operand is 128 x 128 (4 rows x 32 vectors; K = {hi, lo} x {re, im} x 32)
// and whose B operand is 128 x 128: the 32-point DFT matrix in the 2x2 real
// form of complex multiplication, rounded to 16 bits (W_hi, N rows 0-63) and
// its remainder rounded (W_lo, rows 64-127), each repeated for the hi and lo
// halves of K.  Eight MMAs of K = 16 accumulate the FP32 tile
//     columns 0-63:   (X_hi + X_lo) W_hi,   columns 64-127: (X_hi + X_lo) W_lo
// whose two halves summed give all four hi/lo products, which recovers about
// 22 (FP16) or 16 (BF16) significant bits of each operand.
// FP16 operands are scaled per row by a power of two before step 1 (the row's
// largest component into [2^13, 2^14)) and by the fixed 2^-4 before step 2
// (|Z'| <= 32 sqrt(2) 2^14, so the scaled values stay below FP16's maximum);
// BF16 operands are not scaled.  The inverse direction runs as
// conj(F(conj x)); the user scale and the inverse of the operand scales are
// applied at the store.
//
// The kernel is persistent: one 1024-thread CTA per SM holding four
// independent row groups (8 warps each: warp q takes row q % 4 of the group
// and the half q / 4 of its vectors or outputs), one 32 KB A operand and 128
// tensor-memory columns per group, and one B operand and the [c][b] twiddle
// table for the CTA (32 + 8 KB, bulk copies at the start).  A group loops over
// groups of 4 rows; rows are read from and written to global memory directly
// by coalesced per-lane accesses (lane = vector b on the way in, output c on
// the way out), and the group's next rows are prefetched into L2 at the start
// of each iteration.  (Loading them into registers one iteration ahead was
// measured slower: the extra live registers spill at 64 per thread.)  Step
// 1's operand is K-major (a lane writes 16-byte chunks of 8 consecutive a);
// step 2's is MN-major (a lane holds Z'[b][c] for 16 consecutive c, written
// as 16-byte chunks of 8 consecutive c), so no lane exchanges are needed.
// One elected thread per group issues the 8 tcgen05.mma of a step and
// commits them to the group's mbarrier; the group's warps synchronise on a
// named barrier.  Every wait is bounded; on expiry the kernel records a
// status that the next synchronisation reports (E_DEVICE), waits (bounded)
// for MMAs and copies still in flight and frees its tensor memory.
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
constexpr int SPNN = 128;                        // GEMM N: {W_hi, W_lo} x {re, im} x 32
constexpr uint32_t SP_B_LBO = (SPNN / 8) * 128;  // B: bytes between K-adjacent core matrices
constexpr int SP_B_BYTES = 16 * SP_B_LBO;        // 32768
constexpr uint32_t SQ_KS = 128;                  // A: bytes between K-adjacent core matrices
constexpr uint32_t SQ_MS = 2048;                 // A: bytes between M-adjacent core matrices
constexpr int SQ_A_BYTES = 16 * SQ_MS;           // 32768 per group
constexpr int SQG = 4;                           // row groups per CTA
constexpr int SQW = 8;                           // warps per row group
constexpr int SQ_THREADS = SQG * SQW * 32;       // 1024
constexpr int SQ_TMEM_COLS = SQG * SPNN;         // 512
constexpr int SQ_TW_BYTES = 32 * 32 * 8;         // the [c][b] twiddle table
constexpr uint32_t SP_WAIT_LIMIT = 1u << 24;

// byte offset of element (row, k) of a K-major no-swizzle operand made of
// 8-row x 16-byte core matrices: [k/8] (lbo apart) [row/8] (128 apart) [row%8][k%8]
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, uint32_t lbo) {
    return (uint32_t)(k >> 3) * lbo + (uint32_t)((row >> 3) << 7) + (uint32_t)((row & 7) << 4) + (uint32_t)((k & 7) << 1);
}
// A operand element (m, k): K-major for step 1 (core matrix = 8 rows m x 8
// consecutive k), MN-major for step 2 (core matrix = 8 k x 8 consecutive m);
// core matrices SQ_MS apart along m and SQ_KS apart along k in both
__host__ __device__ __forceinline__ uint32_t a_off_k(int m, int k) {
    return (uint32_t)(m >> 3) * SQ_MS + (uint32_t)(k >> 3) * SQ_KS + (uint32_t)((m & 7) << 4) + (uint32_t)((k & 7) << 1);
}
__host__ __device__ __forceinline__ uint32_t a_off_mn(int m, int k) {
    return (uint32_t)(m >> 3) * SQ_MS + (uint32_t)(k >> 3) * SQ_KS + (uint32_t)((k & 7) << 4) + (uint32_t)((m & 7) << 1);
}

struct SplitArgs {
    const float2 *in;
    float2 *out;
    long off_in, vs_in, off_out, vs_out;
    long nvec;
    int inv, has_scale;
    float scale;
    const uint4 *bop;     // B operand, SP_B_BYTES in core-matrix layout
    const float2 *tw;     // [c][b] = s2 exp(-2 pi i bc/1024), c, b < 32 (s2: the step 2 operand scale)
    int *status;          // set to 1 when a barrier wait expired
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

// power of two bringing m (a row's largest component) into [2^13, 2^14)
__device__ __forceinline__ float row_scale(float m) {
    if (!(m > 0.f) || !isfinite(m)) return 1.f;
    return ldexpf(1.f, 13 - ilogbf(m));
}

__device__ __forceinline__ float warp_max(float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

// named barrier of `n` threads; the second form returns the AND of v over them
__device__ __forceinline__ void bar_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" :: "r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ bool bar_and(int id, int n, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r) : "r"((uint32_t)v), "r"(id), "r"(n) : "memory");
    return r != 0;
}

__device__ __forceinline__ void prefetch_l2(const void *p) {
    asm volatile("{\n\t.reg .u64 a;\n\tcvta.to.global.u64 a, %0;\n\tprefetch.global.L2 [a];\n\t}" :: "l"(p));
}

__device__ __forceinline__ void sts128(unsigned char *p, uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(x, y, z, w);
}

// one step into tensor memory at `d`: the 8 K-chunks of 16 (X_hi then X_lo,
// each {re, im} x 32) against B, whose N = 128 columns are W_hi and W_lo side
// by side (the same for both halves of K), so columns 0-63 accumulate
// (X_hi + X_lo) W_hi and columns 64-127 (X_hi + X_lo) W_lo -- all four hi/lo
// products.  da / db are the descriptors of the operands' first K chunks (a
// chunk is 2 * SQ_KS bytes further in A and 2 * SP_B_LBO in B; the address
// field counts 16 bytes)
__device__ __forceinline__ void split_mma(uint32_t d, uint64_t da, uint64_t db, uint32_t idesc) {
#pragma unroll
    for (int k = 0; k < 8; k++)
        tc::mma_f16(d, da + (uint64_t)(k * 2 * SQ_KS / 16), db + (uint64_t)(k * 2 * SP_B_LBO / 16), idesc, k > 0);
}

// the step's result for 8 columns (c or d) from j0 of this lane's row: the
// sum of the W_hi and W_lo halves of the tile
__device__ __forceinline__ void tile_read8(uint32_t lane_addr, int j0, float (&re)[8], float (&im)[8]) {
    float a[8], b[8];
    tc::tmem_ld8(lane_addr + j0, re);
    tc::tmem_ld8(lane_addr + 64 + j0, a);
    tc::tmem_ld8(lane_addr + 32 + j0, im);
    tc::tmem_ld8(lane_addr + 96 + j0, b);
    tc::tmem_ld_wait();
#pragma unroll
    for (int i = 0; i < 8; i++) {
        re[i] += a[i];
        im[i] += b[i];
    }
}

// half h of row `row` (v[i] = x[32 (16h + i) + b], b = lane), conjugated for
// the inverse; rows at or beyond nvec read as zeros
__device__ __forceinline__ void load_half(const SplitArgs &a, long row, int h, int lane, float2 (&v)[16]) {
    const bool live = row < a.nvec;
    const float2 *src = a.in + a.off_in + (live ? row : 0) * a.vs_in + 512 * h + lane;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        float2 c = live ? src[32 * i] : make_float2(0.f, 0.f);
        if (a.inv) c.y = -c.y;
        v[i] = c;
    }
}

// Persistent kernel: gridDim.x CTAs of SQG row groups; group slot grp of CTA
// blk processes the 4-row groups g = grp * gridDim.x + blk, stepping by
// gridDim.x * SQG.  The slot's next rows are prefetched into L2 at the start
// of each iteration.
template <bool BF>
__global__ void __launch_bounds__(SQ_THREADS, 1) k_split1024(const SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bbar, mbar[SQG];
    __shared__ uint32_t tslot;
    __shared__ float smax[SQG][SQW];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int grp = warp / SQW, q = warp % SQW, r = q & 3, h = q >> 2;
    const int gt = tid % (SQW * 32);               // thread index within the group
    const int bar_id = 1 + grp, bar_n = SQW * 32;
    unsigned char *Bsm = smem;
    const float2 *tws = reinterpret_cast<const float2 *>(smem + SP_B_BYTES);
    unsigned char *Asm = smem + SP_B_BYTES + SQ_TW_BYTES + grp * SQ_A_BYTES;
    if (warp == 0) {
        tc::tmem_alloc(&tslot, SQ_TMEM_COLS);
        tc::tmem_relinquish();
    }
    if (tid == 0) {
        for (int g = 0; g < SQG; g++) tc::mbar_init(&mbar[g], 1);
        tc::mbar_init(&bbar, 1);
        tc::mbar_expect_tx(&bbar, SP_B_BYTES + SQ_TW_BYTES);
        tc::bulk_load(Bsm, a.bop, SP_B_BYTES, &bbar);
        tc::bulk_load(smem + SP_B_BYTES, a.tw, SQ_TW_BYTES, &bbar);
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    // the B operand and twiddle copies are waited for after the first rows'
    // loads are issued, so the two overlap
    bool ok = true, b_waited = false;
    const uint32_t tmem = tslot + (uint32_t)(grp * SPNN);
    // this warp's tensor-memory lanes: rows 32r..32r+31 of the group's tile
    const uint32_t lane_addr = tmem + ((uint32_t)(r * 32) << 16);
    const uint32_t idesc1 = tc::idesc_f16(SPM, SPNN, BF ? 1 : 0);
    const uint32_t idesc2 = idesc1 | (1u << 15);  // A MN-major
    const int ngroups = (int)((a.nvec + 3) / 4);  // nvec <= 2^31 (checked by the launcher)
    const int gstep = (int)gridDim.x * SQG;
    const float s2 = BF ? 1.f : 0.0625f;  // folded into a.tw
    uint32_t pending = 2u;  // parity of a committed MMA phase this thread has not seen complete (2: none)
    // slot s = grp * gridDim.x + blockIdx.x takes the groups s, s + gstep, ...:
    // the last, partial round of groups spreads over all CTAs
    for (int g = grp * (int)gridDim.x + (int)blockIdx.x; g < ngroups; g += gstep) {
        const long row = (long)g * 4 + r;
        {
            // the slot's next group into L2: 4 rows x 64 lines of 128 bytes
            const long rn = ((long)g + gstep) * 4 + (gt >> 6);
            if (rn < a.nvec) prefetch_l2(a.in + a.off_in + rn * a.vs_in + (gt & 63) * 16);
        }
        float2 v[16];
        load_half(a, row, h, lane, v);
        if (!BF) {
            float mx = 0.f;
#pragma unroll
            for (int i = 0; i < 16; i++) mx = fmaxf(mx, fmaxf(fabsf(v[i].x), fabsf(v[i].y)));
            mx = warp_max(mx);
            if (lane == 0) smax[grp][q] = mx;
        }
        if (!b_waited) {
            ok = tc::mbar_wait(&bbar, 0, SP_WAIT_LIMIT) && ok;
            b_waited = true;
        }
        ok = bar_and(bar_id, bar_n, ok);
        if (!ok) break;
        const float s1 = BF ? 1.f : row_scale(fmaxf(smax[grp][r], smax[grp][r + 4]));
        // step 1 operand A1[m = 32r + b][k = part*64 + ri*32 + a], K-major
        {
            const int m = 32 * r + lane;
#pragma unroll
            for (int j = 0; j < 2; j++) {
                uint32_t hr[4], hi[4], lr[4], li[4];
#pragma unroll
                for (int t = 0; t < 4; t++) {
                    const float2 e0 = v[8 * j + 2 * t], e1 = v[8 * j + 2 * t + 1];
                    split2<BF>(e0.x * s1, e1.x * s1, hr[t], lr[t]);
                    split2<BF>(e0.y * s1, e1.y * s1, hi[t], li[t]);
                }
                const int ka = 16 * h + 8 * j;
                sts128(Asm + a_off_k(m, ka), hr[0], hr[1], hr[2], hr[3]);
                sts128(Asm + a_off_k(m, 32 + ka), hi[0], hi[1], hi[2], hi[3]);
                sts128(Asm + a_off_k(m, 64 + ka), lr[0], lr[1], lr[2], lr[3]);
                sts128(Asm + a_off_k(m, 96 + ka), li[0], li[1], li[2], li[3]);
            }
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        bar_sync(bar_id, bar_n);
        tc::fence_after_sync();
        if (gt == 0) {
            split_mma(tmem, tc::smem_desc(tc::smem_addr(Asm), SQ_KS, SQ_MS),
                      tc::smem_desc(tc::smem_addr(Bsm), SP_B_LBO, 128), idesc1);
            tc::mma_commit(&mbar[grp]);
        }
        pending = 0u;
        ok = tc::mbar_wait(&mbar[grp], 0, SP_WAIT_LIMIT);
        if (ok) pending = 2u;
        tc::fence_after_sync();
        // step 1 result (lane = b, columns re c | im c for c in half h) times
        // s2 w1024^(bc) as the step 2 operand A2[m = 32r + c][k = part*64 + ri*32 + b], MN-major
#pragma unroll
        for (int j = 0; j < 2; j++) {
            float zr[8], zi[8];
            if (ok) {
                tile_read8(lane_addr, 16 * h + 8 * j, zr, zi);
            } else {
#pragma unroll
                for (int i = 0; i < 8; i++) zr[i] = zi[i] = 0.f;
            }
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const float2 t = tws[(16 * h + 8 * j + i) * 32 + lane];
                const float re = zr[i] * t.x - zi[i] * t.y, im = zr[i] * t.y + zi[i] * t.x;
                zr[i] = re;
                zi[i] = im;
            }
            uint32_t hr[4], hi[4], lr[4], li[4];
#pragma unroll
            for (int t = 0; t < 4; t++) {
                split2<BF>(zr[2 * t], zr[2 * t + 1], hr[t], lr[t]);
                split2<BF>(zi[2 * t], zi[2 * t + 1], hi[t], li[t]);
            }
            const int mc = 32 * r + 16 * h + 8 * j;
            sts128(Asm + a_off_mn(mc, lane), hr[0], hr[1], hr[2], hr[3]);
            sts128(Asm + a_off_mn(mc, 32 + lane), hi[0], hi[1], hi[2], hi[3]);
            sts128(Asm + a_off_mn(mc, 64 + lane), lr[0], lr[1], lr[2], lr[3]);
            sts128(Asm + a_off_mn(mc, 96 + lane), li[0], li[1], li[2], li[3]);
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        ok = bar_and(bar_id, bar_n, ok);
        tc::fence_after_sync();
        if (!ok) break;
        pending = 2u;  // the step 1 products completed (every thread of the group saw it)
        if (gt == 0) {
            split_mma(tmem, tc::smem_desc(tc::smem_addr(Asm), SQ_KS, SQ_MS),
                      tc::smem_desc(tc::smem_addr(Bsm), SP_B_LBO, 128), idesc2);
            tc::mma_commit(&mbar[grp]);
        }
        pending = 1u;
        ok = tc::mbar_wait(&mbar[grp], 1, SP_WAIT_LIMIT);
        tc::fence_after_sync();
        if (ok) {
            pending = 2u;
            // step 2 result: lane = c, columns re d | im d for d in half h -> out[c + 32d]
            const float f = (a.has_scale ? a.scale : 1.f) / (s1 * s2);
            const bool live = row < a.nvec;
            float2 *dst = a.out + a.off_out + (live ? row : 0) * a.vs_out + 512 * h + lane;
#pragma unroll
            for (int j = 0; j < 2; j++) {
                float yr[8], yi[8];
                tile_read8(lane_addr, 16 * h + 8 * j, yr, yi);
                if (live) {
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        float2 o = make_float2(yr[i] * f, yi[i] * f);
                        if (a.inv) o.y = -o.y;
                        dst[32 * (8 * j + i)] = o;
                    }
                }
            }
        }
        // the next iteration's first barrier orders these tensor-memory reads
        // before the next products overwrite the tile
        tc::fence_before_sync();
    }
    // a slot without groups still waits for the B and twiddle copies into the
    // CTA's shared memory before the CTA can end
    if (!b_waited) ok = tc::mbar_wait(&bbar, 0, SP_WAIT_LIMIT) && ok;
    if (!ok) {
        atomicExch(a.status, 1);
        // let MMAs and the B copy still in flight finish (bounded) before the
        // tensor memory and the CTA's shared memory are released
        if (pending < 2u) tc::mbar_wait(&mbar[grp], pending, SP_WAIT_LIMIT);
        tc::mbar_wait(&bbar, 0, SP_WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tslot, SQ_TMEM_COLS);
}

// ---------------------------------------------------------------- host side
// B operand of both steps: row n = pw*64 + ro*32 + c, column k = px*64 +
// ri*32 + a, the real 2x2 form of w32^(ac) = exp(-2 pi i ac/32) (FP64, then
// split): (ro, ri) = (re, re): cos, (re, im): -sin, (im, re): +sin, (im, im):
// cos; rows pw = 0 hold the 16-bit rounding W_hi of each entry, rows pw = 1
// the rounding W_lo of its remainder, the same for both halves px of K (the
// hi and lo parts of the data).
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
                    for (int px = 0; px < 2; px++) {
                        b[core_off(n, px * 64 + ri * 32 + aa, SP_B_LBO) / 2] = hi;
                        b[core_off(64 + n, px * 64 + ri * 32 + aa, SP_B_LBO) / 2] = lo;
                    }
                }
    return b;
}

static std::mutex g_sp_mu;
static void *g_bop[2] = {nullptr, nullptr};
static void *g_tw[2] = {nullptr, nullptr};  // [c][b] twiddles times 2^-4 (FP16 form), times 1 (BF16 form)
static int *g_status = nullptr;

static bool split_tables() {
    if (g_bop[0] && g_bop[1] && g_tw[0] && g_tw[1] && g_status) return true;
    std::vector<uint16_t> b16 = b_operand<false>(), bbf = b_operand<true>();
    std::vector<float> w(2 * 32 * 32), w16(2 * 32 * 32);
    for (int c = 0; c < 32; c++)
        for (int bb = 0; bb < 32; bb++) {
            double ang = -2.0 * 3.14159265358979323846264338327950288 * (double)(bb * c) / SPN;
            w[2 * (c * 32 + bb)] = (float)cos(ang);
            w[2 * (c * 32 + bb) + 1] = (float)sin(ang);
            w16[2 * (c * 32 + bb)] = w[2 * (c * 32 + bb)] * 0.0625f;  // exact: a power of two
            w16[2 * (c * 32 + bb) + 1] = w[2 * (c * 32 + bb) + 1] * 0.0625f;
        }
    g_bop[0] = dmalloc(SP_B_BYTES);
    g_bop[1] = dmalloc(SP_B_BYTES);
    g_tw[0] = dmalloc(w.size() * sizeof(float));
    g_tw[1] = dmalloc(w.size() * sizeof(float));
    g_status = (int *)dmalloc(sizeof(int));
    if (!g_bop[0] || !g_bop[1] || !g_tw[0] || !g_tw[1] || !g_status) return false;
    return cuda_ok(cudaMemcpy(g_bop[0], b16.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_bop[1], bbf.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_tw[0], w16.data(), w16.size() * sizeof(float), cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_tw[1], w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemset(g_status, 0, sizeof(int)), "split status");
}

// true when the split form ran (or failed with an error recorded); false when
// the call does not qualify and the plain kernels should run instead
bool launch_split_f32(const Job &j, cudaStream_t st) {
    if (j.form != JVSIP_FORM_SPLIT_BF16 && j.form != JVSIP_FORM_SPLIT_FP16) return false;
    // the kernel counts groups of 4 rows in 32-bit integers
    if (j.kind != K_C2C || j.prec != P_F32 || j.N != SPN || j.nvec <= 0 || j.nvec > (1L << 31)) return false;
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
    a.tw = (const float2 *)g_tw[bf ? 1 : 0];
    a.status = g_status;
    // operand reads: A chunks start at 2 * k * SQ_KS (k < 8) and span 16
    // core matrices along m (SQ_MS apart) and 2 along k, ending at byte
    // 14 * SQ_KS + 15 * SQ_MS + 2 * SQ_KS - 1 < SQ_A_BYTES of the group's A
    // (whichever of the two descriptor strides is taken along m); B chunks
    // start at 2 * k * SP_B_LBO and span 16 core matrices along n (128 apart)
    // and 2 along k, ending at byte 16 * SP_B_LBO - 1 of B: all inside the
    // operands
    const long ngroups = (j.nvec + 3) / 4;
    Device *d = device();
    long grid = (ngroups + SQG - 1) / SQG;
    if (grid > d->sms) grid = d->sms;
    const size_t smem = SP_B_BYTES + SQ_TW_BYTES + SQG * SQ_A_BYTES;
    static std::atomic<bool> attr[2]{};  // set once per form; concurrent first calls both set it
    if (!attr[bf]) {
        cudaError_t e = bf ? cudaFuncSetAttribute(k_split1024<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                           : cudaFuncSetAttribute(k_split1024<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!cuda_ok(e, "cudaFuncSetAttribute")) return true;
        attr[bf] = true;
    }
    if (bf) k_split1024<true><<<(unsigned)grid, SQ_THREADS, smem, st>>>(a);
    else k_split1024<false><<<(unsigned)grid, SQ_THREADS, smem, st>>>(a);
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
