// nn_kernels.cu -- kernels of the learned warm start: a 3-D U-Net mapping the
// initial field B0 to a grid displacement x(X) - X.  Activations are BF16,
// channels-last ([voxel][channel], voxel = x + nx (y + ny z)), viewed with a
// channel stride so that a concatenation is two views into one buffer.  The
// 3x3x3 convolutions (forward, input gradient, weight gradient) are implicit
// GEMMs on the 5th-generation tensor cores with FP32 accumulation in tensor
// memory (nn_tc.cuh); padding is periodic in x and y and zero in z, as the
// relaxation's boundaries are.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

#include "glemur.h"
#include "gm_internal.h"
#include "nn_tc.cuh"

namespace gmnn {

// ---- tensor-core GEMM check -------------------------------------------------

// D[128 x N] = A[128 x K] . B[N x K]^T with BF16 operands (row-major in global
// memory) and FP32 accumulation in tensor memory; one CTA of 128 threads.
// status[0] is set to 1 when the completion wait gives up.
__global__ void __launch_bounds__(128) k_tc_gemm(const __nv_bfloat16* __restrict__ A,
                                                 const __nv_bfloat16* __restrict__ B, float* __restrict__ D, int N,
                                                 int K, int* status) {
    extern __shared__ __align__(128) unsigned char sm[];
    unsigned char* sA = sm;                               // 128 x K
    unsigned char* sB = sm + 128 * K * 2;                 // N x K
    uint64_t* bar = reinterpret_cast<uint64_t*>(sB + N * K * 2);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int e = tid; e < 128 * K; e += 128) {
        const int r = e / K, k = e % K;
        *reinterpret_cast<__nv_bfloat16*>(sA + kmajor_off(r, k, K)) = A[e];
    }
    for (int e = tid; e < N * K; e += 128) {
        const int r = e / K, k = e % K;
        *reinterpret_cast<__nv_bfloat16*>(sB + kmajor_off(r, k, K)) = B[e];
    }
    if (tid == 0) mbar_init_tc(bar);
    fence_async_smem();
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    if (warp == 0) tmem_alloc(tslot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    if (tid == 0) {
        const uint32_t id = idesc_bf16(128, N);
        for (int kk = 0; kk < K / 16; kk++) {
            const uint64_t ad = smem_desc(sm_addr(sA) + kk * 256, 128, (uint32_t)K * 16);
            const uint64_t bd = smem_desc(sm_addr(sB) + kk * 256, 128, (uint32_t)K * 16);
            mma_bf16(tbase, ad, bd, id, kk > 0);
        }
        mma_commit(bar);
    }
    const bool ok = mbar_wait_tc(bar, 0);
    tc_fence_after();
    if (ok) {
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
#pragma unroll
            for (int q = 0; q < 16; q++) D[(32 * warp + lane) * N + c + q] = v[q];
        }
    } else if (lane == 0) {
        atomicExch(status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tbase, ncols);
}

// ---- convolution: forward and input gradient --------------------------------

struct ConvArgs {
    const __nv_bfloat16* in1; int ld1, c1;   // first input view (channels 0 .. c1-1)
    const __nv_bfloat16* in2; int ld2, c2;   // optional second view (channels c1 .. c1+c2-1)
    const __nv_bfloat16* W;                  // [27][Np][Kc] BF16: rows = output channels, K = input channels
    const float* bias;                       // [Np] or null
    __nv_bfloat16* out; int ldo, co;         // output view (co channels written)
    const __nv_bfloat16* mask; int ldm;      // optional: out *= (mask > 0), mask has co channels
    int relu;
    int nx, ny, nz, xper, yper;
    int Kc, Np;                              // padded input channels (multiple of 16), padded outputs
    int Nt;                                  // output channels per CTA (multiple of 16; blockIdx.y picks the slice)
    int Kch;                                 // input channels per pipeline step (multiple of 16)
    int* status;
    int stall;                               // failure-detection test: wait on an mbarrier nothing arrives on
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Pipeline of the convolution: a step is one tap and one chunk of the input
// channels, all of them up to 96 (one step per tap), else chunks of kConvKc
// (so that the stages stay small enough for two CTAs per SM);
// kConvStages steps of operands are in flight.
constexpr int kConvKc = 64;
constexpr int kConvStages = 4;

// 16-byte asynchronous copy global -> shared (cp.async, L2 only), or 16 zero
// bytes when !valid (source size 0: nothing is read from src).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sm_addr(dst)), "l"(src),
                 "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One CTA: 128 consecutive voxels x one slice of Nt output channels
// (blockIdx.y; all Np when they fit), accumulated over the 27 taps.  The
// operands of a step (the tap's A tile: 128 voxels x one chunk of input
// channels at the tap's offset; and its B tile: the slice's weights for that
// chunk) are copied straight into shared memory with cp.async, kConvStages
// steps ahead, while one thread issues the tensor-core MMAs of the current
// step; a stage is refilled once the MMAs that read it have committed.
__global__ void __launch_bounds__(128) k_conv(const ConvArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    constexpr int S = kConvStages;
    const int Kc = a.Kc, KCH = a.Kch;
    const int n0 = blockIdx.y * a.Nt;                 // first output channel of the slice
    const int Np = min(a.Nt, a.Np - n0);              // channels of this slice (a multiple of 16)
    const int aBytes = 128 * KCH * 2, bBytes = a.Nt * KCH * 2;
    unsigned char* stA = sm;                          // S stages of A, then S stages of B
    unsigned char* stB = sm + S * aBytes;
    // mbarriers: one per stage (MMA commits) and one that nothing arrives on
    // (the failure-detection test waits on it)
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + S * (aBytes + bBytes));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + S + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long V = (long long)a.nx * a.ny * a.nz;
    const long long v = (long long)blockIdx.x * 128 + tid;
    const bool valid = v < V;
    const int vi = valid ? (int)(v % a.nx) : 0;
    const int vj = valid ? (int)((v / a.nx) % a.ny) : 0;
    const int vk = valid ? (int)(v / ((long long)a.nx * a.ny)) : 0;
    const int nk = (Kc + KCH - 1) / KCH;             // channel chunks per tap
    const int T = 27 * nk;                           // steps
    uint32_t ncols = 32;
    while ((int)ncols < Np) ncols <<= 1;
    if (tid == 0)
        for (int q = 0; q <= S; q++) mbar_init_tc(&bars[q]);
    if (warp == 0) tmem_alloc(tslot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t id = idesc_bf16(128, Np);

    // the copies of step q into stage q % S
    auto issue = [&](int q) {
        const int st = q % S;
        const int t = q / nk, kc0 = (q % nk) * KCH, kcw = min(KCH, Kc - kc0);
        const int dk = t / 9 - 1, dj = (t / 3) % 3 - 1, di = t % 3 - 1;
        // A: row tid = this thread's voxel at the tap's offset
        int i = vi + di, j = vj + dj;
        const int k = vk + dk;
        bool in = valid && k >= 0 && k < a.nz && (a.xper || (i >= 0 && i < a.nx)) && (a.yper || (j >= 0 && j < a.ny));
        i = wrap(i, a.nx);
        j = wrap(j, a.ny);
        const long long u = in ? (long long)i + (long long)a.nx * (j + (long long)a.ny * k) : 0;
        unsigned char* dA = stA + st * aBytes;
        for (int c = 0; c < kcw; c += 8) {
            const int cc = kc0 + c;
            const __nv_bfloat16* src = a.in1;
            bool ok8 = in;
            if (cc < a.c1) src = a.in1 + u * a.ld1 + cc;
            else if (cc - a.c1 < a.c2) src = a.in2 + u * a.ld2 + (cc - a.c1);
            else ok8 = false;
            cp_async16(dA + kmajor_off(tid, c, KCH), ok8 ? src : a.in1, ok8);
        }
        // B: the slice's Np x kcw weights of the tap.  A thread copies the 8
        // channels cc, cc + 64, ... (cc = 8 (tid / 16)) of rows tid % 16,
        // tid % 16 + 16, ...: the 8 lanes of a shared-memory store phase write
        // the 8 rows of one core matrix
        const __nv_bfloat16* Wt = a.W + ((size_t)t * a.Np + n0) * Kc + kc0;
        unsigned char* dB = stB + st * bBytes;
        for (int cc = (tid >> 4) * 8; cc < kcw; cc += 64)
            for (int r = tid & 15; r < Np; r += 16)
                cp_async16(dB + kmajor_off(r, cc, KCH), Wt + (size_t)r * Kc + cc, true);
    };

    uint32_t ph[S];
    bool pend[S];                    // a commit on bars[s] not yet waited for
    for (int q = 0; q < S; q++) { ph[q] = 0; pend[q] = false; }
    // failure-detection test: a bounded wait that runs out before any MMA
    bool ok = a.stall ? mbar_wait_tc(&bars[S], 0, 1u << 10) : true;
    if (__syncthreads_and(ok)) {
        for (int q = 0; q < S - 1; q++) {
            if (q < T) issue(q);
            cp_async_commit();
        }
        for (int q = 0; q < T; q++) {
            // refill the stage of step q + S - 1: the MMAs of step q - 1 read it
            const int qn = q + S - 1;
            if (qn < T) {
                const int sn = qn % S;
                if (pend[sn]) {
                    if (!mbar_wait_tc(&bars[sn], ph[sn])) ok = false;
                    ph[sn] ^= 1;
                    pend[sn] = false;
                }
            }
            // after a wait ran out no thread copies into a stage and no MMA is issued
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            if (qn < T) issue(qn);
            cp_async_commit();
            cp_async_wait<S - 1>();                  // step q's copies have landed
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            const int s = q % S;
            if (tid == 0) {
                const int kcw = min(KCH, Kc - (q % nk) * KCH);
                for (int kk = 0; kk < kcw / 16; kk++) {
                    const uint64_t ad = smem_desc(sm_addr(stA + s * aBytes) + kk * 256, 128, (uint32_t)KCH * 16);
                    const uint64_t bd = smem_desc(sm_addr(stB + s * bBytes) + kk * 256, 128, (uint32_t)KCH * 16);
                    mma_bf16(tbase, ad, bd, id, q > 0 || kk > 0);
                }
                mma_commit(&bars[s]);
            }
            pend[s] = true;
        }
    }
    // the copies still in flight, and the commits not yet waited for: bounded
    // waits before the accumulator is read or freed
    cp_async_wait_all();
    for (int q = 0; q < S; q++)
        if (pend[q]) {
            if (!mbar_wait_tc(&bars[q], ph[q])) ok = false;
            ph[q] ^= 1;
        }
    ok = __syncthreads_and(ok);
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < Np; c0 += 16) {
            float acc[16];
            tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, acc);
            if (valid) {
                const long long vv = v;
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int c = n0 + c0 + q;
                    if (c >= a.co) break;
                    float y = acc[q] + (a.bias ? a.bias[c] : 0.f);
                    if (a.relu) y = fmaxf(y, 0.f);
                    if (a.mask && !(__bfloat162float(a.mask[vv * a.ldm + c]) > 0.f)) y = 0.f;
                    a.out[vv * a.ldo + c] = __float2bfloat16_rn(y);
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(a.status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tbase, ncols);
}

// ---- convolution: weight gradient --------------------------------------------

// dW[t][o][i] = sum_v dout[v][o] in[v + off(t)][i] as one GEMM per voxel chunk
// with the 27 taps stacked along M: row m = t Cp + i (Cp = ci rounded up to 8),
// column n = output channel o (N = co rounded up to 16), K = voxels.  Both
// operands are read as they lie in the channels-last buffers: 16 bytes are 8
// channels of one voxel, which is one row of a core matrix of the MN-major
// operand layout, so a copy goes straight from global to shared memory
// (cp.async) with no transpose.
//
// MN-major, no swizzle: a step of kWgKV voxels of an operand with R rows (M or
// N) is kWgKV / 16 slices of 16 voxels, one per MMA (K = 16); slice s holds
// R / 8 x 2 core matrices of 128 bytes (8 voxels x 8 channels), core (rb, h) at
// s R 32 + rb 256 + h 128 bytes.  So neighbouring core matrices along the rows
// are 256 bytes apart (the descriptor's stride-dimension offset) and along K
// 128 bytes apart (its leading-dimension offset).  Read with the two offsets
// exchanged, every address would still fall inside the slice.
constexpr int kWgKV = 64;
constexpr int kWgStages = 4;

__device__ __forceinline__ uint32_t mn_off(int rb, int w, int R) {
    return (uint32_t)((w >> 4) * R * 32 + rb * 256 + (w & 15) * 16);
}

struct WgradArgs {
    const __nv_bfloat16* dout; int ldd, co;  // upstream gradient (channels up to co rounded to 8 readable)
    const __nv_bfloat16* in1; int ld1, c1;   // forward input views
    const __nv_bfloat16* in2; int ld2, c2;
    float* dW;                               // [27][co][ci] FP32, accumulated with atomics
    int ci, Cp;                              // input channels of the weights; rows per tap (ci rounded to 8)
    int N;                                   // MMA columns: co rounded up to 16
    int nx, ny, nz, xper, yper;
    int vchunk;                              // voxels per CTA (multiple of kWgKV)
    int* status;
    int stall;                               // failure-detection test: wait on an mbarrier nothing arrives on
};

// grid = (voxel chunks, row tiles of 128 stacked (tap, channel) rows).  The
// operands of a step (kWgKV voxels: the tile's rows of the input at their taps'
// offsets, and the upstream gradient) are copied kWgStages steps ahead while
// one thread issues the MMAs of the current step; a stage is refilled once the
// MMAs that read it have committed.
__global__ void __launch_bounds__(128) k_conv_wgrad(const WgradArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    constexpr int S = kWgStages, KV = kWgKV;
    const int N = a.N;
    const int aBytes = 128 * KV * 2, bBytes = N * KV * 2;
    unsigned char* stA = sm;                          // S stages of A, then S stages of B
    unsigned char* stB = sm + S * aBytes;
    // mbarriers: one per stage (MMA commits) and one that nothing arrives on
    // (the failure-detection test waits on it)
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + S * (aBytes + bBytes));
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + S + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = 128 * blockIdx.y;                  // first stacked row of this CTA
    const int V = a.nx * a.ny * a.nz;                 // < 2^31 (checked by the host)
    const int v0 = blockIdx.x * a.vchunk;
    const int nv = min(V - v0, a.vchunk);             // voxels of this chunk
    const int T = (nv + KV - 1) / KV;                 // steps
    const int w = tid & (KV - 1);                     // this thread's voxel within a step
    const int cpb = a.Cp >> 3;                        // 8-channel groups per tap
    // this thread's 8 row blocks of A (rb = tid / 64 + 2 r): the tap's offset
    // packed as (di + 1) | (dj + 1) << 2 | (dk + 1) << 4 (-1: a row beyond the
    // 27 taps or the input's channels, zero-filled), and the source view from
    // the block's first channel, with its channel stride
    int tapo[8], ldr[8];
    const __nv_bfloat16* srcr[8];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const int g = (m0 >> 3) + (tid >> 6) + 2 * r;
        const int t = g / cpb, c = (g - t * cpb) * 8;
        tapo[r] = t < 27 ? (t % 3) | (((t / 3) % 3) << 2) | ((t / 9) << 4) : -1;
        srcr[r] = a.in1;
        ldr[r] = 0;
        if (c < a.c1) { srcr[r] = a.in1 + c; ldr[r] = a.ld1; }
        else if (c - a.c1 < a.c2) { srcr[r] = a.in2 + (c - a.c1); ldr[r] = a.ld2; }
        else tapo[r] = -1;
    }
    // the coordinates of this thread's voxel v0 + kWgKV q + w of the next step
    // to issue, advanced by kWgKV = si + nx (sj + ny sk) voxels per step
    int vi, vj, vk;
    {
        const int v = v0 + w;
        vi = v % a.nx;
        vj = (v / a.nx) % a.ny;
        vk = v / (a.nx * a.ny);
    }
    const int si = KV % a.nx, sj = (KV / a.nx) % a.ny, sk = KV / (a.nx * a.ny);
    uint32_t ncols = 32;
    while ((int)ncols < N) ncols <<= 1;
    if (tid == 0)
        for (int q = 0; q <= S; q++) mbar_init_tc(&bars[q]);
    if (warp == 0) tmem_alloc(tslot, ncols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    // A and B both MN-major (transpose bits 15 and 16)
    const uint32_t id = idesc_bf16(128, N) | (1u << 15) | (1u << 16);

    // the copies of step q into stage q % S (called for q = 0, 1, 2, ... in turn)
    auto issue = [&](int q) {
        const int st = q % S;
        const int vl = q * KV + w;
        const bool vin = vl < nv;
        const int v = v0 + vl;
        unsigned char* dA = stA + st * aBytes;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int to = tapo[r];
            int ii = vi + (to & 3) - 1, jj = vj + ((to >> 2) & 3) - 1;
            const int kk = vk + (to >> 4) - 1;
            const bool ok = vin && to >= 0 && kk >= 0 && kk < a.nz && (a.xper || (ii >= 0 && ii < a.nx)) &&
                            (a.yper || (jj >= 0 && jj < a.ny));
            ii = wrap(ii, a.nx);
            jj = wrap(jj, a.ny);
            const int u = ok ? ii + a.nx * (jj + a.ny * kk) : 0;
            cp_async16(dA + mn_off((tid >> 6) + 2 * r, w, 128), ok ? srcr[r] + (size_t)u * ldr[r] : a.in1, ok);
        }
        unsigned char* dB = stB + st * bBytes;
        for (int nb = tid >> 6; nb < N / 8; nb += 2) {
            const bool ok = vin && nb * 8 < a.co;
            cp_async16(dB + mn_off(nb, w, N), ok ? a.dout + (size_t)v * a.ldd + nb * 8 : a.dout, ok);
        }
        // the next step's voxel
        vi += si;
        const int cx = vi >= a.nx;
        vi -= cx ? a.nx : 0;
        vj += sj + cx;
        const int cy = vj >= a.ny;
        vj -= cy ? a.ny : 0;
        vk += sk + cy;
    };

    uint32_t ph[S];
    bool pend[S];                    // a commit on bars[s] not yet waited for
    for (int q = 0; q < S; q++) { ph[q] = 0; pend[q] = false; }
    // failure-detection test: a bounded wait that runs out before any MMA
    bool ok = a.stall ? mbar_wait_tc(&bars[S], 0, 1u << 10) : true;
    if (__syncthreads_and(ok)) {
        for (int q = 0; q < S - 1; q++) {
            if (q < T) issue(q);
            cp_async_commit();
        }
        for (int q = 0; q < T; q++) {
            // refill the stage of step q + S - 1: the MMAs of step q - 1 read it
            const int qn = q + S - 1;
            if (qn < T) {
                const int sn = qn % S;
                if (pend[sn]) {
                    if (!mbar_wait_tc(&bars[sn], ph[sn])) ok = false;
                    ph[sn] ^= 1;
                    pend[sn] = false;
                }
            }
            // after a wait ran out no thread copies into a stage and no MMA is issued
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            if (qn < T) issue(qn);
            cp_async_commit();
            cp_async_wait<S - 1>();                  // step q's copies have landed
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            const int s = q % S;
            if (tid == 0) {
                for (int kk = 0; kk < KV / 16; kk++) {
                    const uint64_t ad = smem_desc(sm_addr(stA + s * aBytes) + kk * 128 * 32, 128, 256);
                    const uint64_t bd = smem_desc(sm_addr(stB + s * bBytes) + kk * N * 32, 128, 256);
                    mma_bf16(tbase, ad, bd, id, q > 0 || kk > 0);
                }
                mma_commit(&bars[s]);
            }
            pend[s] = true;
        }
    }
    // the copies still in flight, and the commits not yet waited for: bounded
    // waits before the accumulator is read or freed
    cp_async_wait_all();
    for (int q = 0; q < S; q++)
        if (pend[q]) {
            if (!mbar_wait_tc(&bars[q], ph[q])) ok = false;
            ph[q] ^= 1;
        }
    ok = __syncthreads_and(ok);
    tc_fence_after();
    // this thread's row: tap t, input channel ich
    const int g = m0 + 32 * warp + lane;
    const int t = g / a.Cp, ich = g - t * a.Cp;
    const bool mine = t < 27 && ich < a.ci;
    if (ok && T > 0) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float acc[16];
            tmem_ld16(tbase + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, acc);
            if (mine) {
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int o = c0 + q;
                    if (o < a.co) atomicAdd(&a.dW[((size_t)t * a.co + o) * a.ci + ich], acc[q]);
                }
            }
        }
    } else if (!ok && tid == 0) {
        atomicExch(a.status, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tbase, ncols);
}

// ---- elementwise and resampling kernels ---------------------------------------

// Sum over voxels of an upstream gradient per channel (bias gradient).
__global__ void k_bias_grad(const __nv_bfloat16* __restrict__ d, int ld, int c, long long V, float* __restrict__ db) {
    __shared__ float red[256];
    const int ch = blockIdx.y;
    float s = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
        s += __bfloat162float(d[v * ld + ch]);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(&db[ch], red[0]);
}

// 2x2x2 average pooling (forward) and its adjoint (backward: each child gets
// 1/8 of the parent's gradient).  Fine grid (nx, ny, nz), coarse (nx/2, ...).
__global__ void k_pool(const __nv_bfloat16* __restrict__ in, int ldi, __nv_bfloat16* __restrict__ out, int ldo, int c,
                       int nx, int ny, int nz, int backward, int accumulate) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const long long Vc = (long long)cx * cy * cz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < Vc * c; q += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(q % c);
        const long long vc = q / c;
        const int i = (int)(vc % cx), j = (int)((vc / cx) % cy), k = (int)(vc / ((long long)cx * cy));
        if (!backward) {
            float s = 0.f;
            for (int d = 0; d < 8; d++) {
                const long long vf = (2 * i + (d & 1)) + (long long)nx * ((2 * j + ((d >> 1) & 1)) + (long long)ny * (2 * k + (d >> 2)));
                s += __bfloat162float(in[vf * ldi + ch]);
            }
            out[vc * ldo + ch] = __float2bfloat16_rn(0.125f * s);
        } else {
            // in = coarse gradient, out = fine gradient
            const float g = 0.125f * __bfloat162float(in[vc * ldi + ch]);
            for (int d = 0; d < 8; d++) {
                const long long vf = (2 * i + (d & 1)) + (long long)nx * ((2 * j + ((d >> 1) & 1)) + (long long)ny * (2 * k + (d >> 2)));
                const float o = accumulate ? __bfloat162float(out[vf * ldo + ch]) : 0.f;
                out[vf * ldo + ch] = __float2bfloat16_rn(o + g);
            }
        }
    }
}

// Nearest-neighbour 2x upsampling (forward) and its adjoint (backward: the sum
// of the 8 children).  Coarse grid (nx/2, ...), fine (nx, ny, nz).
__global__ void k_upsample(const __nv_bfloat16* __restrict__ in, int ldi, __nv_bfloat16* __restrict__ out, int ldo,
                           int c, int nx, int ny, int nz, int backward) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const long long Vc = (long long)cx * cy * cz;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < Vc * c; q += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(q % c);
        const long long vc = q / c;
        const int i = (int)(vc % cx), j = (int)((vc / cx) % cy), k = (int)(vc / ((long long)cx * cy));
        if (!backward) {
            const __nv_bfloat16 x = in[vc * ldi + ch];
            for (int d = 0; d < 8; d++) {
                const long long vf = (2 * i + (d & 1)) + (long long)nx * ((2 * j + ((d >> 1) & 1)) + (long long)ny * (2 * k + (d >> 2)));
                out[vf * ldo + ch] = x;
            }
        } else {
            // in = fine gradient, out = coarse gradient
            float s = 0.f;
            for (int d = 0; d < 8; d++) {
                const long long vf = (2 * i + (d & 1)) + (long long)nx * ((2 * j + ((d >> 1) & 1)) + (long long)ny * (2 * k + (d >> 2)));
                s += __bfloat162float(in[vf * ldi + ch]);
            }
            out[vc * ldo + ch] = __float2bfloat16_rn(s);
        }
    }
}

// d *= (y > 0): the gradient through a ReLU from its output.
__global__ void k_relu_bwd(__nv_bfloat16* __restrict__ d, int ldd, const __nv_bfloat16* __restrict__ y, int ldy, int c,
                           long long V) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < V * c; q += (long long)gridDim.x * blockDim.x) {
        const long long v = q / c;
        const int ch = (int)(q % c);
        if (!(__bfloat162float(y[v * ldy + ch]) > 0.f)) d[v * ldd + ch] = __float2bfloat16_rn(0.f);
    }
}

// Masked mean-square error of the 3 output channels against the target
// (FP32, [V][3]); planes k = 0 and nz-1 are excluded (their displacement is
// imposed to be zero).  Writes the gradient (BF16) and adds the loss sum.
// A training sample moved by a symmetry of the periodic cross-section: the
// value at cell (i, j) is read at the source cell u = (i + sx) mod nx,
// v = (j + sy) mod ny, then (sym & 4) u <-> v, (sym & 2) v -> ny - 1 - v,
// (sym & 1) u -> nx - 1 - u; a vector's x, y components are transformed as the
// positions (x negated for bit 1, y for bit 2, then swapped for bit 4), so
// the field and the displacement stay a solution pair of the relaxation (the
// force J x B transforms as a polar vector under reflections).
__device__ __forceinline__ void sym_source(int i, int j, int nx, int ny, int sx, int sy, int sym, int* is, int* js) {
    int u = (i + sx) % nx, v = (j + sy) % ny;
    if (sym & 4) { const int w = u; u = v; v = w; }
    if (sym & 2) v = ny - 1 - v;
    if (sym & 1) u = nx - 1 - u;
    *is = u;
    *js = v;
}
__device__ __forceinline__ void sym_vector(int sym, float* vx, float* vy) {
    if (sym & 1) *vx = -*vx;
    if (sym & 2) *vy = -*vy;
    if (sym & 4) { const float w = *vx; *vx = *vy; *vy = w; }
}

__global__ void k_mse(const __nv_bfloat16* __restrict__ y, int ldy, const float* __restrict__ tgt,
                      __nv_bfloat16* __restrict__ dy, int lddy, int nx, int ny, int nz, float scale,
                      float* __restrict__ loss, int sx, int sy, int sym) {
    __shared__ float red[256];
    const long long V = (long long)nx * ny * nz;
    float s = 0.f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long long)nx * ny));
        const bool in = k > 0 && k < nz - 1;
        int is, js;
        sym_source(i, j, nx, ny, sx, sy, sym, &is, &js);
        const long long vt = (long long)is + (long long)nx * (js + (long long)ny * k);
        float t[3] = {tgt[3 * vt], tgt[3 * vt + 1], tgt[3 * vt + 2]};
        sym_vector(sym, &t[0], &t[1]);
        for (int c = 0; c < 3; c++) {
            const float e = in ? __bfloat162float(y[v * ldy + c]) - t[c] : 0.f;
            s += e * e;
            dy[v * lddy + c] = __float2bfloat16_rn(2.f * scale * e);
        }
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0] * scale);
}

// Adam on FP32 master weights W[27][co][ci] and b[co]; then the BF16 operand
// layouts: Wf[27][Npo][Kci] (forward: rows = outputs) and Wb[27][Npi][Kco]
// (input gradient: taps flipped, rows = inputs).
__global__ void k_adam(float* __restrict__ W, float* __restrict__ mW, float* __restrict__ vW,
                       const float* __restrict__ gW, float* __restrict__ b, float* __restrict__ mb,
                       float* __restrict__ vb, const float* __restrict__ gb, int co, int ci, float lr, float b1,
                       float b2, float c1, float c2, float eps, __nv_bfloat16* __restrict__ Wf, int Npo, int Kci,
                       __nv_bfloat16* __restrict__ Wb, int Npi, int Kco, float* __restrict__ bpad, int step) {
    const long long n = 27LL * co * ci;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n + co; q += (long long)gridDim.x * blockDim.x) {
        if (q < n) {
            float w = W[q];
            if (step) {
                const float g = gW[q];
                const float m = b1 * mW[q] + (1 - b1) * g, v = b2 * vW[q] + (1 - b2) * g * g;
                mW[q] = m;
                vW[q] = v;
                w -= lr * (m / c1) / (sqrtf(v / c2) + eps);
                W[q] = w;
            }
            const int t = (int)(q / ((long long)co * ci)), o = (int)((q / ci) % co), i = (int)(q % ci);
            const __nv_bfloat16 wb = __float2bfloat16_rn(w);
            Wf[((size_t)t * Npo + o) * Kci + i] = wb;
            Wb[((size_t)(26 - t) * Npi + i) * Kco + o] = wb;
        } else {
            const int o = (int)(q - n);
            float x = b[o];
            if (step) {
                const float g = gb[o];
                const float m = b1 * mb[o] + (1 - b1) * g, v = b2 * vb[o] + (1 - b2) * g * g;
                mb[o] = m;
                vb[o] = v;
                x -= lr * (m / c1) / (sqrtf(v / c2) + eps);
                b[o] = x;
            }
            bpad[o] = x;
        }
    }
}

// Input channels (B0x, B0y, B0z - 1) of the inner points, from the ghosted
// AoS B0 of the reference layout (REAL T); ld channels, the rest zero.
// The sample is moved by a symmetry of the periodic cross-section (sym_source,
// sym_vector): whole-cell translations, mirrors and the x <-> y swap, used to
// augment training data.
template <typename T>
__global__ void k_input(const T* __restrict__ B0, int nx, int ny, int nz, __nv_bfloat16* __restrict__ x, int ld,
                        int sx, int sy, int sym) {
    const long long V = (long long)nx * ny * nz;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long long)nx * ny));
        int is, js;
        sym_source(i, j, nx, ny, sx, sy, sym, &is, &js);
        const long long g = (long long)(is + 1) + (long long)(nx + 2) * ((js + 1) + (long long)(ny + 2) * (k + 1));
        float b[3] = {(float)B0[3 * g], (float)B0[3 * g + 1], (float)B0[3 * g + 2] - 1.f};
        sym_vector(sym, &b[0], &b[1]);
        for (int c = 0; c < ld; c++) x[v * ld + c] = __float2bfloat16_rn(c < 3 ? b[c] : 0.f);
    }
}

// ---- the warm-start grid: displacement -> smoothed -> positions ------------

// Displacement channels 0..2 of a network output (BF16, [V][ld]) computed on
// the input translated by (sx, sy) (gm_nn_input), moved back to the grid's
// own cells and weighted: d(i, j, k) = w y((i - sx) mod nx, (j - sy) mod ny, k),
// added to d unless `first`.
__global__ void k_wg_acc(const __nv_bfloat16* __restrict__ y, int ld, int nx, int ny, int nz, int sx, int sy, float w,
                         int first, float* __restrict__ d) {
    const long long V = (long long)nx * ny * nz;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny);
        const long long k = v / ((long long)nx * ny);
        const int is = (i - sx + nx) % nx, js = (j - sy + ny) % ny;
        const long long u = is + (long long)nx * (js + (long long)ny * k);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float val = w * __bfloat162float(y[u * ld + c]);
            d[3 * v + c] = first ? val : d[3 * v + c] + val;
        }
    }
}

// One 3x3x3 box-filter pass, periodic in x / y as selected, zero beyond the
// z range: out(i, j, k) = (1/27) sum of the 27 neighbours.
__global__ void k_wg_box(const float* __restrict__ in, float* __restrict__ out, int nx, int ny, int nz, int xper,
                         int yper) {
    const long long V = (long long)nx * ny * nz;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(v % nx), j = (int)((v / nx) % ny), k = (int)(v / ((long long)nx * ny));
        float acc[3] = {0.f, 0.f, 0.f};
        for (int dk = -1; dk <= 1; dk++) {
            const int kk = k + dk;
            if (kk < 0 || kk >= nz) continue;
            for (int dj = -1; dj <= 1; dj++) {
                int jj = j + dj;
                if (jj < 0 || jj >= ny) {
                    if (!yper) continue;
                    jj = (jj + ny) % ny;
                }
                for (int di = -1; di <= 1; di++) {
                    int ii = i + di;
                    if (ii < 0 || ii >= nx) {
                        if (!xper) continue;
                        ii = (ii + nx) % nx;
                    }
                    const float* q = in + 3 * (ii + (long long)nx * (jj + (long long)ny * kk));
                    acc[0] += q[0]; acc[1] += q[1]; acc[2] += q[2];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 3; c++) out[3 * v + c] = acc[c] * (1.f / 27.f);
    }
}

// Positions of the warm grid in the reference layout (ghosted AoS): the
// identity grid xid plus the displacement (in grid spacings) at the inner
// points, the first and last inner z-planes held; periodic x / y ghosts are
// the images of the opposite inner points shifted by -/+ (L + d) (x first,
// then y, so corners carry both shifts); other ghosts keep xid.
template <typename T>
__global__ void k_wg_grid(const float* __restrict__ d, const T* __restrict__ xid, T* __restrict__ xb, int nx, int ny,
                          int nz, int xper, int yper, double dx, double dy, double dz, double Lx, double Ly) {
    const long long G = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < G; g += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(g % (nx + 2)), j = (int)((g / (nx + 2)) % (ny + 2));
        const int k = (int)(g / ((long long)(nx + 2) * (ny + 2)));
        int is = i, js = j;
        double sx = 0, sy = 0;
        if (xper && i == 0) { is = nx; sx = -(Lx + dx); }
        if (xper && i == nx + 1) { is = 1; sx = Lx + dx; }
        if (yper && j == 0) { js = ny; sy = -(Ly + dy); }
        if (yper && j == ny + 1) { js = 1; sy = Ly + dy; }
        const long long gs = is + (long long)(nx + 2) * (js + (long long)(ny + 2) * k);
        double x[3] = {(double)xid[3 * gs], (double)xid[3 * gs + 1], (double)xid[3 * gs + 2]};
        if (is >= 1 && is <= nx && js >= 1 && js <= ny && k >= 2 && k <= nz - 1) {
            const float* q = d + 3 * ((is - 1) + (long long)nx * ((js - 1) + (long long)ny * (k - 1)));
            x[0] += (double)q[0] * dx;
            x[1] += (double)q[1] * dy;
            x[2] += (double)q[2] * dz;
        }
        x[0] += sx;
        x[1] += sy;
        xb[3 * g] = (T)x[0];
        xb[3 * g + 1] = (T)x[1];
        xb[3 * g + 2] = (T)x[2];
    }
}

static unsigned nb(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 152 * 16 ? 152 * 16 : b));
}

}  // namespace gmnn

using gmnn::ConvArgs;
using gmnn::WgradArgs;

extern "C" {

int gm_nn_tc_gemm_check(const void* A, const void* B, float* D, int N, int K, int* status) {
    if (!A || !B || !D || !status) return gm::fail(GM_EPARAM, "gm_nn_tc_gemm_check: null argument");
    if (N < 16 || N > 256 || N % 16 || K < 16 || K > 256 || K % 16)
        return gm::fail(GM_EPARAM, "gm_nn_tc_gemm_check: N and K must be multiples of 16 in [16, 256]");
    const size_t smem = (size_t)(128 + N) * K * 2 + 16;
    cudaError_t e = cudaFuncSetAttribute(gmnn::k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    gmnn::k_tc_gemm<<<1, 128, smem>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, N, K, status);
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("k_tc_gemm: ") + cudaGetErrorString(e));
    return GM_OK;
}

static int check_view_align(const void* p, int ld, const char* what) {
    if (p && ((reinterpret_cast<uintptr_t>(p) & 15) || (ld % 8)))
        return gm::fail(GM_EPARAM, std::string(what) + ": views must start on 16 bytes with a channel stride that is a multiple of 8");
    return GM_OK;
}

namespace {
// failure-detection test hook (gm_nn_debug_stall): read when a convolution is launched
int g_nn_stall = 0;
}  // namespace

int gm_nn_debug_stall(int on) {
    g_nn_stall = on ? 1 : 0;
    return GM_OK;
}

int gm_nn_conv(const void* in1, int ld1, int c1, const void* in2, int ld2, int c2, const void* W, const float* bias,
               void* out, int ldo, int co, const void* mask, int ldm, int relu, int nx, int ny, int nz, int xper,
               int yper, int Kc, int Np, int* status, void* stream) {
    if (!in1 || !W || !out || !status) return gm::fail(GM_EPARAM, "gm_nn_conv: null argument");
    if (Kc % 16 || Kc < 16 || Kc > 256 || Np % 16 || Np < 16 || Np > 256 || c1 + (in2 ? c2 : 0) > Kc || co > Np ||
        c1 % 8)
        return gm::fail(GM_EPARAM, "gm_nn_conv: channel counts out of range");
    // output channels per CTA: all of them when the operand stages fit the
    // shared memory, else the widest multiple of 16 that fits (slices in
    // blockIdx.y)
    // input channels per pipeline step: all of them up to 96 (one step per
    // tap), else kConvKc
    const int Kch = Kc <= 96 ? Kc : gmnn::kConvKc;
    auto conv_smem = [Kch](int nt) { return (size_t)gmnn::kConvStages * (128 + nt) * Kch * 2 + 64; };
    int Nt = Np;
    while (Nt > 16 && conv_smem(Nt) > 200 * 1024) Nt -= 16;
    if (conv_smem(Nt) > 200 * 1024) return gm::fail(GM_EPARAM, "gm_nn_conv: channel counts out of range");
    int rc;
    if ((rc = check_view_align(in1, ld1, "gm_nn_conv in1")) || (rc = check_view_align(in2, ld2, "gm_nn_conv in2")))
        return rc;
    ConvArgs a;
    a.in1 = (const __nv_bfloat16*)in1; a.ld1 = ld1; a.c1 = c1;
    a.in2 = (const __nv_bfloat16*)in2; a.ld2 = ld2; a.c2 = in2 ? c2 : 0;
    a.W = (const __nv_bfloat16*)W; a.bias = bias;
    a.out = (__nv_bfloat16*)out; a.ldo = ldo; a.co = co;
    a.mask = (const __nv_bfloat16*)mask; a.ldm = ldm; a.relu = relu;
    a.nx = nx; a.ny = ny; a.nz = nz; a.xper = xper; a.yper = yper; a.Kc = Kc; a.Np = Np; a.Nt = Nt; a.Kch = Kch; a.status = status;
    a.stall = g_nn_stall;
    const size_t smem = conv_smem(Nt);
    cudaError_t e = cudaFuncSetAttribute(gmnn::k_conv, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    const long long V = (long long)nx * ny * nz;
    const dim3 grid((unsigned)((V + 127) / 128), (unsigned)((Np + Nt - 1) / Nt));
    gmnn::k_conv<<<grid, 128, smem, (cudaStream_t)stream>>>(a);
    e = cudaGetLastError();
    return e == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, std::string("k_conv: ") + cudaGetErrorString(e));
}

int gm_nn_conv_wgrad(const void* dout, int ldd, int co, const void* in1, int ld1, int c1, const void* in2, int ld2,
                     int c2, float* dW, int ci, int nx, int ny, int nz, int xper, int yper, int vchunk, int* status,
                     void* stream) {
    if (!dout || !in1 || !dW || !status) return gm::fail(GM_EPARAM, "gm_nn_conv_wgrad: null argument");
    const long long V = (long long)nx * ny * nz;
    if (ci > c1 + (in2 ? c2 : 0) || ci < 1 || co > 256 || co < 1 || vchunk < 0 || vchunk % gmnn::kWgKV || c1 % 8 ||
        nx < 1 || ny < 1 || nz < 1 || V >= (1ll << 31))
        return gm::fail(GM_EPARAM, "gm_nn_conv_wgrad: channel counts, grid or chunk out of range");
    int rc;
    if ((rc = check_view_align(dout, ldd, "gm_nn_conv_wgrad dout")) ||
        (rc = check_view_align(in1, ld1, "gm_nn_conv_wgrad in1")) || (rc = check_view_align(in2, ld2, "gm_nn_conv_wgrad in2")))
        return rc;
    WgradArgs a;
    a.dout = (const __nv_bfloat16*)dout; a.ldd = ldd; a.co = co;
    a.in1 = (const __nv_bfloat16*)in1; a.ld1 = ld1; a.c1 = c1;
    a.in2 = (const __nv_bfloat16*)in2; a.ld2 = ld2; a.c2 = in2 ? c2 : 0;
    a.dW = dW; a.ci = ci; a.Cp = (ci + 7) / 8 * 8; a.N = (co + 15) / 16 * 16;
    a.nx = nx; a.ny = ny; a.nz = nz; a.xper = xper; a.yper = yper;
    a.status = status;
    a.stall = g_nn_stall;
    const int tiles = (27 * a.Cp + 127) / 128;
    if (vchunk == 0) {
        // about four CTAs per SM over the grid, at least 8 steps each: fewer,
        // longer CTAs cost fewer accumulator flushes (atomics)
        int dev = 0, nsm = 152;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        const long long chunks = (4LL * nsm + tiles - 1) / tiles;
        long long vc = (V + chunks - 1) / chunks;
        vc = (vc + gmnn::kWgKV - 1) / gmnn::kWgKV * gmnn::kWgKV;
        vchunk = (int)(vc < 8 * gmnn::kWgKV ? 8 * gmnn::kWgKV : vc);
    }
    a.vchunk = vchunk;
    const size_t smem = (size_t)gmnn::kWgStages * (128 + a.N) * gmnn::kWgKV * 2 + 8 * (gmnn::kWgStages + 1) + 16;
    cudaError_t e = cudaFuncSetAttribute(gmnn::k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return gm::fail(GM_ECUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
    const dim3 grid((unsigned)((V + vchunk - 1) / vchunk), (unsigned)tiles);
    gmnn::k_conv_wgrad<<<grid, 128, smem, (cudaStream_t)stream>>>(a);
    e = cudaGetLastError();
    return e == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, std::string("k_conv_wgrad: ") + cudaGetErrorString(e));
}

int gm_nn_bias_grad(const void* d, int ld, int c, long long V, float* db, void* stream) {
    gmnn::k_bias_grad<<<dim3(gmnn::nb(V) > 64 ? 64 : gmnn::nb(V), c), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)d, ld, c, V, db);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_bias_grad");
}

int gm_nn_pool(const void* in, int ldi, void* out, int ldo, int c, int nx, int ny, int nz, int backward,
               int accumulate, void* stream) {
    if (nx % 2 || ny % 2 || nz % 2) return gm::fail(GM_EPARAM, "gm_nn_pool: grid sizes must be even");
    const long long n = (long long)(nx / 2) * (ny / 2) * (nz / 2) * c;
    gmnn::k_pool<<<gmnn::nb(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, ldi, (__nv_bfloat16*)out,
                                                                 ldo, c, nx, ny, nz, backward, accumulate);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_pool");
}

int gm_nn_upsample(const void* in, int ldi, void* out, int ldo, int c, int nx, int ny, int nz, int backward,
                   void* stream) {
    if (nx % 2 || ny % 2 || nz % 2) return gm::fail(GM_EPARAM, "gm_nn_upsample: grid sizes must be even");
    const long long n = (long long)(nx / 2) * (ny / 2) * (nz / 2) * c;
    gmnn::k_upsample<<<gmnn::nb(n), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)in, ldi,
                                                                     (__nv_bfloat16*)out, ldo, c, nx, ny, nz, backward);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_upsample");
}

int gm_nn_input(const void* B0, int precision, int nx, int ny, int nz, void* x, int ld, int sx, int sy, int sym,
                void* stream) {
    if (sx < 0 || sx >= nx || sy < 0 || sy >= ny) return gm::fail(GM_EPARAM, "gm_nn_input: shift out of range");
    if (sym < 0 || sym > 7 || ((sym & 4) && nx != ny))
        return gm::fail(GM_EPARAM, "gm_nn_input: sym is 0..7, and the x <-> y swap needs nx == ny");
    const long long V = (long long)nx * ny * nz;
    if (precision == 32)
        gmnn::k_input<float><<<gmnn::nb(V), 256, 0, (cudaStream_t)stream>>>((const float*)B0, nx, ny, nz,
                                                                              (__nv_bfloat16*)x, ld, sx, sy, sym);
    else
        gmnn::k_input<double><<<gmnn::nb(V), 256, 0, (cudaStream_t)stream>>>((const double*)B0, nx, ny, nz,
                                                                               (__nv_bfloat16*)x, ld, sx, sy, sym);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_input");
}

int gm_nn_disp_accumulate(const void* y, int ldy, int nx, int ny, int nz, int sx, int sy, float w, int first,
                          float* d, void* stream) {
    if (!y || !d || ldy < 3 || sx < 0 || sx >= nx || sy < 0 || sy >= ny)
        return gm::fail(GM_EPARAM, "gm_nn_disp_accumulate: bad argument");
    const long long V = (long long)nx * ny * nz;
    gmnn::k_wg_acc<<<gmnn::nb(V), 256, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)y, ldy, nx, ny, nz, sx, sy, w,
                                                                   first, d);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "gm_nn_disp_accumulate");
}

int gm_nn_warm_grid(const float* d, const gm_params* p, int passes, const void* xid, float* scratch, void* xb,
                    void* stream) {
    if (!d || !p || !xid || !scratch || !xb || passes < 0)
        return gm::fail(GM_EPARAM, "gm_nn_warm_grid: bad argument");
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const long long V = (long long)nx * ny * nz, G = (long long)(nx + 2) * (ny + 2) * (nz + 2);
    cudaStream_t s = (cudaStream_t)stream;
    float* a = scratch;
    float* b = scratch + 3 * V;
    if (cudaMemcpyAsync(a, d, 3 * V * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return gm::fail(GM_ECUDA, "gm_nn_warm_grid: copy of the displacement failed");
    for (int q = 0; q < passes; q++) {
        gmnn::k_wg_box<<<gmnn::nb(V), 256, 0, s>>>(a, b, nx, ny, nz, p->xPeri, p->yPeri);
        float* t = a; a = b; b = t;
    }
    if (p->precision == 32)
        gmnn::k_wg_grid<float><<<gmnn::nb(G), 256, 0, s>>>(a, (const float*)xid, (float*)xb, nx, ny, nz, p->xPeri,
                                                            p->yPeri, p->dx, p->dy, p->dz, p->Lx, p->Ly);
    else
        gmnn::k_wg_grid<double><<<gmnn::nb(G), 256, 0, s>>>(a, (const double*)xid, (double*)xb, nx, ny, nz, p->xPeri,
                                                             p->yPeri, p->dx, p->dy, p->dz, p->Lx, p->Ly);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "gm_nn_warm_grid");
}

int gm_nn_zero(void* p, size_t bytes, void* stream) {
    const cudaError_t e = cudaMemsetAsync(p, 0, bytes, (cudaStream_t)stream);
    return e == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
}

int gm_nn_relu_bwd(void* d, int ldd, const void* y, int ldy, int c, long long V, void* stream) {
    gmnn::k_relu_bwd<<<gmnn::nb(V * c), 256, 0, (cudaStream_t)stream>>>((__nv_bfloat16*)d, ldd,
                                                                         (const __nv_bfloat16*)y, ldy, c, V);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_relu_bwd");
}

int gm_nn_mse(const void* y, int ldy, const float* tgt, void* dy, int lddy, int nx, int ny, int nz, float scale,
              float* loss, int sx, int sy, int sym, void* stream) {
    if (sx < 0 || sx >= nx || sy < 0 || sy >= ny) return gm::fail(GM_EPARAM, "gm_nn_mse: shift out of range");
    if (sym < 0 || sym > 7 || ((sym & 4) && nx != ny))
        return gm::fail(GM_EPARAM, "gm_nn_mse: sym is 0..7, and the x <-> y swap needs nx == ny");
    const long long V = (long long)nx * ny * nz;
    gmnn::k_mse<<<gmnn::nb(V) > 256 ? 256 : gmnn::nb(V), 256, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16*)y, ldy, tgt, (__nv_bfloat16*)dy, lddy, nx, ny, nz, scale, loss, sx, sy, sym);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_mse");
}

int gm_nn_adam(float* W, float* mW, float* vW, const float* gW, float* b, float* mb, float* vb, const float* gb, int co,
               int ci, float lr, float b1, float b2, int t, float eps, void* Wf, int Npo, int Kci, void* Wb, int Npi,
               int Kco, float* bpad, void* stream) {
    const float c1 = t > 0 ? 1.f - powf(b1, (float)t) : 1.f, c2 = t > 0 ? 1.f - powf(b2, (float)t) : 1.f;
    gmnn::k_adam<<<gmnn::nb(27LL * co * ci + co), 256, 0, (cudaStream_t)stream>>>(
        W, mW, vW, gW, b, mb, vb, gb, co, ci, lr, b1, b2, c1, c2, eps, (__nv_bfloat16*)Wf, Npo, Kci,
        (__nv_bfloat16*)Wb, Npi, Kco, bpad, t > 0 ? 1 : 0);
    return cudaGetLastError() == cudaSuccess ? GM_OK : gm::fail(GM_ECUDA, "k_adam");
}

}  // extern "C"
