// jv_split.cu -- precision form: 1024-point rows as two tensor-core DFT
// products with hi/lo-split 16-bit operands and FP32 accumulation.
//
// A row x (n = 32a + b) is a 32 x 32 matrix X[a][b].  Its DFT is the
// four-step  Z = F32^T-applied over a,  Z'[c][b] = Z[c][b] * w1024^(bc),
// X[c + 32d] = sum_b Z'[c][b] w32^(bd).  Each step is a real GEMM of a
// 128 x 192 A operand (4 rows x 32 vectors, K = {hi, lo, hi} x {re, im} x 32)
// with a 64 x 192 B operand (the 32-point DFT matrix, {hi, hi, lo} x the 2x2
// real form of complex multiplication), so the three products
// hi*hi + lo*hi + hi*lo recover about 22 (FP16) or 16 (BF16) significant
// bits of each operand while the tensor core accumulates in FP32.  FP16
// operands are scaled per row by a power of two before the split (so their
// range fits FP16); BF16 operands are not scaled.  The inverse direction runs
// as conj(F(conj x)); the user scale is applied at the store.
//
// Per CTA: 128 threads, one warp per row; TMEM holds the two 128 x 64 FP32
// accumulators (128 columns); one elected thread issues 12 tcgen05.mma per
// step and commits them to an mbarrier the CTA waits on with a bounded loop.
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

constexpr int SPN = 1024;            // transform length of the form
constexpr int SPM = 128;             // GEMM M: 4 rows x 32
constexpr int SPK = 192;             // GEMM K
constexpr int SPNN = 64;             // GEMM N
constexpr int SP_A_BYTES = SPM * SPK * 2;
constexpr int SP_B_BYTES = SPNN * SPK * 2;
constexpr uint32_t SP_WAIT_LIMIT = 1u << 24;

// byte offset of element (row, k) of a K-major operand with `rows` rows laid out as
// no-swizzle core matrices: [k/8][row/8][row%8][k%8]
__host__ __device__ __forceinline__ uint32_t core_off(int row, int k, int rows) {
    return (uint32_t)((((k >> 3) * (rows >> 3) + (row >> 3)) << 7) + ((row & 7) << 4) + ((k & 7) << 1));
}

struct SplitArgs {
    const float2 *in;
    float2 *out;
    long off_in, vs_in, off_out, vs_out;
    long nvec;
    int inv, has_scale;
    float scale;
    const uint4 *bop;     // B operand, SP_B_BYTES in core-matrix layout
    const float2 *w1024;  // exp(-2 pi i m/1024)
    int *status;          // set to 1 when a barrier wait expired
};

template <bool BF>
__device__ __forceinline__ uint16_t to16(float x) {
    if (BF) return __bfloat16_as_ushort(__float2bfloat16_rn(x));
    return __half_as_ushort(__float2half_rn(x));
}
template <bool BF>
__device__ __forceinline__ float from16(uint16_t h) {
    if (BF) return __bfloat162float(__ushort_as_bfloat16(h));
    return __half2float(__ushort_as_half(h));
}

// power-of-two scale bringing the warp's largest magnitude into [2^13, 2^14)
__device__ __forceinline__ float warp_scale(float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (!(m > 0.f) || !isfinite(m)) return 1.f;
    int e = ilogbf(m);
    return ldexpf(1.f, 13 - e);
}

template <bool BF>
__global__ void __launch_bounds__(128) k_split1024(const SplitArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *Asm = smem;                     // 48 KiB, 1024-aligned
    unsigned char *Bsm = smem + SP_A_BYTES;        // 24 KiB
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, w = tid >> 5, l = tid & 31;
    const long row = (long)blockIdx.x * 4 + w;
    const bool live = row < a.nvec;

    if (w == 0) {
        tc::tmem_alloc(&tslot, 128);
        tc::tmem_relinquish();
    }
    if (tid == 0) tc::mbar_init(&mbar, 1);
    // B operand (constant per plan) into shared memory
    {
        uint4 *dst = reinterpret_cast<uint4 *>(Bsm);
        for (int i = tid; i < SP_B_BYTES / 16; i += 128) dst[i] = __ldg(&a.bop[i]);
    }
    // ---- step 1 operand: thread (w, l) owns vector b = l of row w: x[32a + l], a < 32
    float2 v[32];
    const float2 *src = a.in + a.off_in + (live ? row : 0) * a.vs_in;
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < 32; i++) {
        float2 c = live ? src[32 * i + l] : make_float2(0.f, 0.f);
        if (a.inv) c.y = -c.y;
        v[i] = c;
        mx = fmaxf(mx, fmaxf(fabsf(c.x), fabsf(c.y)));
    }
    const float s1 = BF ? 1.f : warp_scale(mx);
    {
        const int m = w * 32 + l;
        // k = part*64 + ri*32 + a; parts: X_hi, X_lo, X_hi
#pragma unroll
        for (int ab = 0; ab < 4; ab++) {
            uint16_t hr[8], hi_[8], lr[8], li[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                float xr = v[ab * 8 + q].x * s1, xi = v[ab * 8 + q].y * s1;
                hr[q] = to16<BF>(xr);
                hi_[q] = to16<BF>(xi);
                lr[q] = to16<BF>(xr - from16<BF>(hr[q]));
                li[q] = to16<BF>(xi - from16<BF>(hi_[q]));
            }
            uint4 phr, phi, plr, pli;
            phr.x = hr[0] | (uint32_t)hr[1] << 16; phr.y = hr[2] | (uint32_t)hr[3] << 16;
            phr.z = hr[4] | (uint32_t)hr[5] << 16; phr.w = hr[6] | (uint32_t)hr[7] << 16;
            phi.x = hi_[0] | (uint32_t)hi_[1] << 16; phi.y = hi_[2] | (uint32_t)hi_[3] << 16;
            phi.z = hi_[4] | (uint32_t)hi_[5] << 16; phi.w = hi_[6] | (uint32_t)hi_[7] << 16;
            plr.x = lr[0] | (uint32_t)lr[1] << 16; plr.y = lr[2] | (uint32_t)lr[3] << 16;
            plr.z = lr[4] | (uint32_t)lr[5] << 16; plr.w = lr[6] | (uint32_t)lr[7] << 16;
            pli.x = li[0] | (uint32_t)li[1] << 16; pli.y = li[2] | (uint32_t)li[3] << 16;
            pli.z = li[4] | (uint32_t)li[5] << 16; pli.w = li[6] | (uint32_t)li[7] << 16;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 0 + ab * 8, SPM)) = phr;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 32 + ab * 8, SPM)) = phi;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 64 + ab * 8, SPM)) = plr;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 96 + ab * 8, SPM)) = pli;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 128 + ab * 8, SPM)) = phr;
            *reinterpret_cast<uint4 *>(Asm + core_off(m, 160 + ab * 8, SPM)) = phi;
        }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tbase = tslot;
    const uint32_t idesc = tc::idesc_f16(SPM, SPNN, BF ? 1 : 0);
    const uint32_t a0 = tc::smem_addr(Asm), b0 = tc::smem_addr(Bsm);
    const uint32_t lbo_a = (SPM / 8) * 128, lbo_b = (SPNN / 8) * 128, sbo = 128;
    if (tid == 0) {
#pragma unroll 1
        for (int kc = 0; kc < SPK / 16; kc++)
            tc::mma_f16(tbase, tc::smem_desc(a0 + kc * 2 * lbo_a, lbo_a, sbo), tc::smem_desc(b0 + kc * 2 * lbo_b, lbo_b, sbo),
                        idesc, kc > 0);
        tc::mma_commit(&mbar);
    }
    bool ok = tc::mbar_wait(&mbar, 0, SP_WAIT_LIMIT);
    ok = __syncthreads_and(ok);
    uint32_t pending = ok ? 2u : 0u;  // phase still outstanding if a wait gives up
    tc::fence_after_sync();
    // ---- step 1 result: lane (w, l) = (row, b), columns re c | im c
    float zr[32], zi[32];
    const uint32_t lane_base = tbase + ((uint32_t)(w * 32) << 16);
    if (ok) {
        float t[16];
        tc::tmem_ld16(lane_base + 0, t);
#pragma unroll
        for (int i = 0; i < 16; i++) zr[i] = t[i];
        tc::tmem_ld16(lane_base + 16, t);
#pragma unroll
        for (int i = 0; i < 16; i++) zr[16 + i] = t[i];
        tc::tmem_ld16(lane_base + 32, t);
#pragma unroll
        for (int i = 0; i < 16; i++) zi[i] = t[i];
        tc::tmem_ld16(lane_base + 48, t);
#pragma unroll
        for (int i = 0; i < 16; i++) zi[16 + i] = t[i];
        tc::tmem_ld_wait();
    }
    // twiddle w1024^(b c), b = l
    mx = 0.f;
#pragma unroll
    for (int c = 0; c < 32; c++) {
        float2 tw = __ldg(&a.w1024[(l * c) & (SPN - 1)]);
        float r = zr[c] * tw.x - zi[c] * tw.y, i = zr[c] * tw.y + zi[c] * tw.x;
        zr[c] = r;
        zi[c] = i;
        mx = fmaxf(mx, fmaxf(fabsf(r), fabsf(i)));
    }
    const float s2 = BF ? 1.f : warp_scale(mx);
    // ---- step 2 operand: A2[(w, c)][part*64 + ri*32 + b], b = l (overwrites A after step 1)
#pragma unroll
    for (int c = 0; c < 32; c++) {
        const int m = w * 32 + c;
        float xr = zr[c] * s2, xi = zi[c] * s2;
        uint16_t hr = to16<BF>(xr), hi_ = to16<BF>(xi);
        uint16_t lr = to16<BF>(xr - from16<BF>(hr)), li = to16<BF>(xi - from16<BF>(hi_));
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, l, SPM)) = hr;
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, 32 + l, SPM)) = hi_;
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, 64 + l, SPM)) = lr;
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, 96 + l, SPM)) = li;
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, 128 + l, SPM)) = hr;
        *reinterpret_cast<uint16_t *>(Asm + core_off(m, 160 + l, SPM)) = hi_;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && ok) {
#pragma unroll 1
        for (int kc = 0; kc < SPK / 16; kc++)
            tc::mma_f16(tbase + SPNN, tc::smem_desc(a0 + kc * 2 * lbo_a, lbo_a, sbo),
                        tc::smem_desc(b0 + kc * 2 * lbo_b, lbo_b, sbo), idesc, kc > 0);
        tc::mma_commit(&mbar);
    }
    if (ok) {
        ok = tc::mbar_wait(&mbar, 1, SP_WAIT_LIMIT);
        ok = __syncthreads_and(ok);
        pending = ok ? 2u : 1u;
    }
    tc::fence_after_sync();
    // ---- step 2 result: lane (w, l) = (row, c = l), columns re d | im d -> out[c + 32 d]
    if (ok) {
        float yr[32], yi[32], t[16];
        tc::tmem_ld16(lane_base + SPNN + 0, t);
#pragma unroll
        for (int i = 0; i < 16; i++) yr[i] = t[i];
        tc::tmem_ld16(lane_base + SPNN + 16, t);
#pragma unroll
        for (int i = 0; i < 16; i++) yr[16 + i] = t[i];
        tc::tmem_ld16(lane_base + SPNN + 32, t);
#pragma unroll
        for (int i = 0; i < 16; i++) yi[i] = t[i];
        tc::tmem_ld16(lane_base + SPNN + 48, t);
#pragma unroll
        for (int i = 0; i < 16; i++) yi[16 + i] = t[i];
        tc::tmem_ld_wait();
        if (live) {
            const float f = (a.has_scale ? a.scale : 1.f) / (s1 * s2);
            float2 *dst = a.out + a.off_out + row * a.vs_out;
#pragma unroll
            for (int d = 0; d < 32; d++) {
                float2 o = make_float2(yr[d] * f, yi[d] * f);
                if (a.inv) o.y = -o.y;
                dst[l + 32 * d] = o;
            }
        }
    } else {
        if (tid == 0) atomicExch(a.status, 1);
        // let MMAs still in flight finish (bounded) before the tensor memory is freed
        if (pending < 2u) tc::mbar_wait(&mbar, pending, SP_WAIT_LIMIT);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_dealloc(tbase, 128);
}

// ---------------------------------------------------------------- host side
// B operand of both steps: row n = ro*32 + c, column k = part*64 + ri*32 + a,
// the real 2x2 form of w32^(ac) = exp(-2 pi i ac/32) (FP64, then split):
// (ro, ri) = (re, re): cos, (re, im): +sin, (im, re): -sin, (im, im): cos;
// parts {hi, hi, lo} pair with the A parts {hi, lo, hi}.
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
                    const uint16_t parts[3] = {hi, hi, lo};
                    for (int part = 0; part < 3; part++) {
                        int k = part * 64 + ri * 32 + aa;
                        b[core_off(n, k, SPNN) / 2] = parts[part];
                    }
                }
    return b;
}

static std::mutex g_sp_mu;
static void *g_bop[2] = {nullptr, nullptr};
static void *g_w1024 = nullptr;
static int *g_status = nullptr;

static bool split_tables() {
    if (g_bop[0] && g_bop[1] && g_w1024 && g_status) return true;
    std::vector<uint16_t> b16 = b_operand<false>(), bbf = b_operand<true>();
    std::vector<float> w(2 * SPN);
    for (int m = 0; m < SPN; m++) {
        double ang = -2.0 * 3.14159265358979323846264338327950288 * (double)m / SPN;
        w[2 * m] = (float)cos(ang);
        w[2 * m + 1] = (float)sin(ang);
    }
    g_bop[0] = dmalloc(SP_B_BYTES);
    g_bop[1] = dmalloc(SP_B_BYTES);
    g_w1024 = dmalloc(w.size() * sizeof(float));
    g_status = (int *)dmalloc(sizeof(int));
    if (!g_bop[0] || !g_bop[1] || !g_w1024 || !g_status) return false;
    return cuda_ok(cudaMemcpy(g_bop[0], b16.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_bop[1], bbf.data(), SP_B_BYTES, cudaMemcpyHostToDevice), "split tables") &&
           cuda_ok(cudaMemcpy(g_w1024, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice), "split tables") &&
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
    a.w1024 = (const float2 *)g_w1024;
    a.status = g_status;
    // operand reads end at byte 49151 of A and 24575 of B (K step = LBO,
    // M/N step = SBO): inside the two operands
    const size_t smem = SP_A_BYTES + SP_B_BYTES;
    static bool attr[2] = {false, false};
    if (!attr[bf]) {
        cudaError_t e = bf ? cudaFuncSetAttribute(k_split1024<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                           : cudaFuncSetAttribute(k_split1024<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!cuda_ok(e, "cudaFuncSetAttribute")) return true;
        attr[bf] = true;
    }
    const long grid = (j.nvec + 3) / 4;
    if (bf) k_split1024<true><<<(unsigned)grid, 128, smem, st>>>(a);
    else k_split1024<false><<<(unsigned)grid, 128, smem, st>>>(a);
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
