// tg3_fused.cu -- projection and split-bf16 scoring in one persistent kernel.
//
// D[dOff + r nT + t] = alpha * sum_k P_r[k] A''_t[k] + norm_r for every
// rotation r and translation t of every particle, where P_r is the Fourier
// slice of the particle's class volume at rotation r (trilinear, Friedel
// mirrored: Projector::project, src/Projector.cpp:356-374) and A''_t the
// particle's shifted, CTF- and sigma-weighted data (k_shift_bank).  The same
// contraction as k_project + k_gemm_bf16x3, but the slices never leave the SM:
// they are gathered straight into the shared-memory A operand of the tensor
// cores, so neither the 8 B per sample of the slice bank nor its re-read
// touches HBM.
//
// Work item: 128 rotations (the UMMA M) of one particle.  One CTA per SM takes
// items from an atomic counter.  Per item the CTA sweeps the particle's pixels
// in K blocks of 32 pixels (64 bf16 = one 128-byte swizzle row):
//   - all 32 warps gather: a lane pair serves one pixel of the block for 8
//     rotation rows (lane half h reads slab z0 + h of the 64-byte corner
//     block), then writes the hi and lo bf16 of its real (h = 0) or imaginary
//     (h = 1) part into the block's A stage in the 128-byte-swizzled K-major
//     layout UMMA reads, and accumulates the row norm sigRcp ctf^2 |P|^2;
//   - each warp fences its writes to the async proxy and arrives on the
//     stage's A barrier; thread 0, the single issuer of every MMA, commit and
//     copy of the CTA (so each commit covers all earlier MMAs), waits for the
//     stage's A barrier and B tile (TMA, issued S - 1 blocks ahead), issues
//     the 3 x 4 UMMAs 128 x N x 16 (Ah Bh + Ah Bl + Al Bh), commits to the
//     stage's empty barrier and starts the TMA of a later block.  The other
//     warps run up to S - 1 blocks ahead of warp 0;
//   - after the last block all warps read the tensor-memory accumulator
//     (warp w: lanes 32 (w % 4) .., columns 16 (w / 4) ..) and write D.
// The CTAs resident at once hold the first items of consecutive particles and
// sweep the pixels in the same order, so the volume blocks of one pixel band
// stay in L2 while every rotation of those particles reads them.
//
// Every mbarrier wait is bounded; a wait that runs out records TG3 flag bit 4
// and sets the CTA's abort word, after which no thread waits again: the CTA
// leaves its block loop, lets its own copies and MMAs land (short bounded
// waits) and frees its tensor memory before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg3_internal.cuh"
#include "tg3_tcgen05.cuh"

namespace tg3 {

namespace {

using namespace tc;

constexpr int FU_WARPS = 32;
constexpr int FU_THREADS = FU_WARPS * 32;
constexpr int FU_M = 128;            // rotation rows per item (UMMA M)
constexpr int FU_BK = 32;            // bf16 elements per K block (one 64-byte row)
constexpr int FU_PIX = FU_BK / 2;    // complex pixels per K block
constexpr int FU_ROWS = 4;           // rotation rows of a lane pair per block
constexpr int FU_U = 2;              // rows whose corner loads are in flight together

struct FusedParams {
    float4* const* volTable;
    int vdim, pf;
    const float* mf;                 // [rows][9] FP32 rotation matrices
    const FusedParticle* part;
    const int* itemOff;              // [nP + 1] first item of every particle
    int nP, nItems;
    FusedPixels pix[kMaxClasses];
    const float* sigRcp;
    const float* ctf;
    float* D;
    float alpha;
    int ntile;                       // rows of a B tile (multiple of 16, <= 256)
    int tmemCols;
    int stages;
    int* flag;
    int* counter;
};

// Byte offset of byte b of row r in a K-major tile of 64-byte rows with the
// 64-byte swizzle (the layout of a TMA SWIZZLE_64B box and of UMMA operands
// described by umma_desc_sw64): 16-byte chunk index XOR ((row / 2) mod 4).
__device__ __forceinline__ uint32_t swz64(int r, int b)
{
    return (uint32_t)((r >> 3) * 512 + (r & 7) * 64 +
                      ((((b >> 4) ^ ((r >> 1) & 3)) << 4) | (b & 15)));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void st_bf16(uint8_t* p, __nv_bfloat16 v)
{
    *reinterpret_cast<__nv_bfloat16*>(p) = v;
}

// The current item, published in shared memory by thread 0 and read where
// used (keeps its pointers out of the registers of the gather loop).
struct ItemDesc {
    const float4* vol;
    const int* iCol;
    const int* iRow;
    const float* sg;
    const float* cf;
    float* drow0;          // D row r0 of the item
    int K, nkb, nRows, ntileI, transRow, nT;
};

__global__ void __launch_bounds__(FU_THREADS, 1)
k_fused_bf16x3(const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
               const __grid_constant__ FusedParams p)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    const int aBytes = FU_M * FU_BK * 2;              // 8 KB per plane
    const int bBytes = p.ntile * FU_BK * 2;           // ntile x 64 B per plane
    const int stageBytes = 2 * aBytes + 2 * bBytes;   // a multiple of 2048
    int* tx = reinterpret_cast<int*>(smem + S * stageBytes);
    int* ty = tx + (p.vdim / 2 + 1);
    int* tz = ty + p.vdim;
    float* mrot = reinterpret_cast<float*>(tz + p.vdim);   // [128][9]
    float* nrmS = mrot + FU_M * 9;                         // [128]
    // row-norm partials of every lane pair: [4 rows j][32 warps][16 pairs]
    float* nacc = nrmS + FU_M;
    uint64_t* bars = reinterpret_cast<uint64_t*>(
        (reinterpret_cast<uintptr_t>(nacc + FU_ROWS * FU_WARPS * 16) + 7) & ~(uintptr_t)7);
    uint64_t* aFull = bars;            // [S] one arrival per warp
    uint64_t* bFull = bars + 4;        // [S] TMA bytes of the B tile
    uint64_t* empty = bars + 8;        // [S] MMAs of the stage complete
    uint64_t* accum = bars + 12;       // the item's accumulator complete
    uint64_t* drain = bars + 13;       // teardown after an abort
    int* misc = reinterpret_cast<int*>(bars + 14);  // [0] abort, [2 + it % 2] item
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(misc + 4);
    ItemDesc* sIt = reinterpret_cast<ItemDesc*>(
        (reinterpret_cast<uintptr_t>(tmemSlot + 1) + 15) & ~(uintptr_t)15);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int h = lane & 1;
    const int pib = lane >> 1;                       // this pair's pixel within a block
    const int rbase = warp;                          // this pair's rows: warp + 32 j
    const int colByte = 4 * pib + 2 * h;             // its bf16 within a 64-byte row

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(aFull + s, FU_WARPS);
            mbar_init(bFull + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accum, 1);
        mbar_init(drain, 1);
        misc[0] = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fill_brick_tables(p.vdim, tx, ty, tz);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmemSlot)),
                     "r"(p.tmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;
    const int half = p.vdim / 2;
    const float fpf = (float)p.pf;

    uint32_t g = 0;           // K blocks this CTA has started (stage slot and phase)
    uint32_t done = 0;        // items finished (accumulator phase)
    bool aborted = false;
    bool mmaPending = false;  // this CTA may have MMAs in flight (abort path)
    for (uint32_t it = 0;; it++) {
        // the item index alternates between two slots, so thread 0 never
        // overwrites one another warp may still be about to read
        if (threadIdx.x == 0) misc[2 + (it & 1)] = atomicAdd(p.counter, 1);
        __syncthreads();
        const int item = misc[2 + (it & 1)];
        if (item >= p.nItems) break;
        int lo = 0, hi = p.nP;   // itemOff[lo] <= item < itemOff[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (p.itemOff[mid] <= item) lo = mid;
            else hi = mid;
        }
        const FusedParticle P = p.part[lo];
        const int r0 = (item - p.itemOff[lo]) * FU_M;
        const int nRows = min(FU_M, P.nR - r0);
        const float4* __restrict__ vol =
            (P.cls >= 0 && P.cls < kMaxClasses) ? p.volTable[P.cls] : nullptr;
        if (!vol || nRows <= 0) {
            // unknown class (or an empty item): record it and leave its rows unwritten
            if (threadIdx.x == 0) atomicOr(p.flag, 8);
            continue;   // uniform: every thread saw the same item
        }
        if (threadIdx.x == 0) {
            const FusedPixels& px = p.pix[P.cls];
            ItemDesc d;
            d.vol = vol;
            d.iCol = px.iCol;
            d.iRow = px.iRow;
            d.sg = p.sigRcp + P.sgOff;
            d.cf = p.ctf + P.sgOff;
            d.drow0 = p.D + P.dOff + (size_t)r0 * P.nT;
            d.K = px.K;
            d.nkb = px.Kp / FU_BK;
            d.nRows = nRows;
            d.ntileI = (P.nT + 15) / 16 * 16;
            d.transRow = P.transRow;
            d.nT = P.nT;
            *sIt = d;
        }
        for (int i = threadIdx.x; i < nRows * 9; i += blockDim.x)
            mrot[i] = p.mf[(size_t)(P.rowOff + r0) * 9 + i];
        __syncthreads();
        // B tiles of the item's first S - 1 blocks; every stage is free here
        // (the previous item's MMAs completed before its epilogue).
        if (threadIdx.x == 0) {
            for (int kb = 0; kb < S - 1 && kb < sIt->nkb; kb++) {
                const int s = (g + kb) % S;
                uint8_t* st = smem + s * stageBytes;
                mbar_expect_tx(bFull + s, 2 * bBytes);
                tma_load_2d(st + 2 * aBytes, &tmBh, bFull + s, kb * FU_BK, sIt->transRow);
                tma_load_2d(st + 2 * aBytes + bBytes, &tmBl, bFull + s, kb * FU_BK, sIt->transRow);
            }
        }
        const int nkb = sIt->nkb;
        float nacc_r[FU_ROWS];
#pragma unroll
        for (int j = 0; j < FU_ROWS; j++) nacc_r[j] = 0.f;
        volatile int* abortp = misc;
        bool bad = false;
        for (int kb = 0; kb < nkb; kb++, g++) {
            const int s = g % S;
            const uint32_t use = g / S;
            uint8_t* st = smem + s * stageBytes;
            // the stage's previous MMAs (block g - S) must have read it
            int ok = !*abortp;
            if (ok && use > 0 && lane == 0) ok = mbar_wait(empty + s, (use - 1) & 1, kWaitBudget);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) {
                    atomicOr(p.flag, 4);
                    *abortp = 1;
                }
                bad = true;
                break;   // warp-uniform; the item end is a CTA-wide meeting point
            }
            const int pg = kb * FU_PIX + pib;
            const bool pv = pg < sIt->K;
            const int pq = pv ? pg : 0;
            const float a = (float)sIt->iCol[pq] * fpf, b = (float)sIt->iRow[pq] * fpf;
            const float w2 = pv ? sIt->sg[pq] * sIt->cf[pq] * sIt->cf[pq] : 0.f;
            const int nRows = sIt->nRows;
            const float4* __restrict__ vol = sIt->vol;
#pragma unroll
            for (int j0 = 0; j0 < FU_ROWS; j0 += FU_U) {
                float fw[FU_U][3];
                bool cj[FU_U];
                float4 c[FU_U][2];
#pragma unroll
                for (int u = 0; u < FU_U; u++) {
                    const int r = rbase + 32 * (j0 + u);
                    const float* mm = mrot + 9 * min(r, nRows - 1);
                    float x = mm[0] * a + mm[1] * b;
                    float y = mm[3] * a + mm[4] * b;
                    float z = mm[6] * a + mm[7] * b;
                    cj[u] = x < 0.f;
                    if (cj[u]) { x = -x; y = -y; z = -z; }
                    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
                    fw[u][0] = x - xf;
                    fw[u][1] = y - yf;
                    fw[u][2] = z - zf;
                    const unsigned blk = (unsigned)(tx[(int)xf] + ty[(int)yf + half] +
                                                    tz[(int)zf + half]);
                    const float4* e = vol + 4 * (size_t)blk + 2 * h;
                    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                        : "=f"(c[u][0].x), "=f"(c[u][0].y), "=f"(c[u][0].z), "=f"(c[u][0].w),
                          "=f"(c[u][1].x), "=f"(c[u][1].y), "=f"(c[u][1].z), "=f"(c[u][1].w)
                        : "l"(e));
                }
#pragma unroll
                for (int u = 0; u < FU_U; u++) {
                    const float fx = fw[u][0], fy = fw[u][1], fz = fw[u][2];
                    const float wz = h ? fz : 1.f - fz;
                    const float wx0 = 1.f - fx, wx1 = fx;
                    const float wy0 = (1.f - fy) * wz, wy1 = fy * wz;
                    float re = c[u][0].x * (wx0 * wy0) + c[u][0].z * (wx1 * wy0);
                    float im = c[u][0].y * (wx0 * wy0) + c[u][0].w * (wx1 * wy0);
                    re += c[u][1].x * (wx0 * wy1) + c[u][1].z * (wx1 * wy1);
                    im += c[u][1].y * (wx0 * wy1) + c[u][1].w * (wx1 * wy1);
                    re += __shfl_xor_sync(0xffffffffu, re, 1);
                    im += __shfl_xor_sync(0xffffffffu, im, 1);
                    const int r = rbase + 32 * (j0 + u);
                    float v = 0.f;
                    if (pv && r < nRows) {
                        if (cj[u]) im = -im;
                        v = h ? im : re;
                        if (h == 0) nacc_r[j0 + u] = fmaf(w2, re * re + im * im, nacc_r[j0 + u]);
                    }
                    const __nv_bfloat16 vh = __float2bfloat16_rn(v);
                    const __nv_bfloat16 vl = __float2bfloat16_rn(v - __bfloat162float(vh));
                    const uint32_t o = swz64(r, colByte);
                    st_bf16(st + o, vh);
                    st_bf16(st + aBytes + o, vl);
                }
            }
            // publish the stage to the tensor cores
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(aFull + s);
            if (threadIdx.x == 0) {
                // the CTA's issuer: A written by all warps, B tile landed
                bool ok2 = !*abortp && mbar_wait(aFull + s, use & 1, kWaitBudget) &&
                           mbar_wait(bFull + s, use & 1, kWaitBudget);
                if (ok2) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t idesc = umma_idesc(FU_M, sIt->ntileI);
                    const uint32_t ah = smem_u32(st), al = smem_u32(st + aBytes);
                    const uint32_t bh = smem_u32(st + 2 * aBytes);
                    const uint32_t bl = smem_u32(st + 2 * aBytes + bBytes);
#pragma unroll
                    for (int kk = 0; kk < FU_BK / 16; kk++) {
                        const uint32_t off = kk * 32;
                        umma_bf16(tmem, umma_desc_sw64(ah + off), umma_desc_sw64(bh + off), idesc,
                                  (kb | kk) != 0);
                        umma_bf16(tmem, umma_desc_sw64(ah + off), umma_desc_sw64(bl + off), idesc, 1);
                        umma_bf16(tmem, umma_desc_sw64(al + off), umma_desc_sw64(bh + off), idesc, 1);
                    }
                    umma_commit(empty + s);
                    if (kb == nkb - 1) umma_commit(accum);
                    // B tile of block kb + S - 1 into the stage block g - 1 used
                    const int kn = kb + S - 1;
                    if (kn < nkb) {
                        const int s2 = (g + S - 1) % S;
                        if (g >= 1) ok2 = mbar_wait(empty + s2, ((g - 1) / S) & 1, kWaitBudget);
                        if (ok2) {
                            uint8_t* st2 = smem + s2 * stageBytes;
                            mbar_expect_tx(bFull + s2, 2 * bBytes);
                            tma_load_2d(st2 + 2 * aBytes, &tmBh, bFull + s2, kn * FU_BK,
                                        sIt->transRow);
                            tma_load_2d(st2 + 2 * aBytes + bBytes, &tmBl, bFull + s2,
                                        kn * FU_BK, sIt->transRow);
                        }
                    }
                }
                if (!ok2) {
                    atomicOr(p.flag, 4);
                    *abortp = 1;
                }
            }
            __syncwarp();
        }
        mmaPending = true;
        // ---- the item's accumulator, then its norms and likelihoods
        int okAcc = !bad && !*abortp;
        if (lane == 0 && okAcc) okAcc = mbar_wait(accum, done & 1, kWaitBudget);
        okAcc = __shfl_sync(0xffffffffu, okAcc, 0);
        if (h == 0) {
#pragma unroll
            for (int j = 0; j < FU_ROWS; j++) nacc[(j * FU_WARPS + warp) * 16 + (lane >> 1)] = nacc_r[j];
        }
        const bool ok = __syncthreads_and(okAcc && !*abortp) != 0;
        if (ok) mmaPending = false;
        if (threadIdx.x < FU_M) {
            // row r's partials: the 16 pairs of warp r % 32, in order
            const int r = threadIdx.x, j = r >> 5, w = r & 31;
            const float* a = nacc + (j * FU_WARPS + w) * 16;
            float sum = 0.f;
            for (int i = 0; i < 16; i++) sum += a[i];
            nrmS[r] = sum;
        }
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (ok) {
            const int qd = warp & 3;
            const int ntileI = sIt->ntileI, nT = sIt->nT;
            for (int c0 = (warp >> 2) * 16; c0 < ntileI; c0 += (FU_WARPS / 4) * 16) {
                float v[16];
                tmem_ld16(tmem + ((uint32_t)(32 * qd) << 16) + (uint32_t)c0, v);
                const int rl = 32 * qd + lane;
                if (rl < sIt->nRows) {
                    float* drow = sIt->drow0 + (size_t)rl * nT;
                    const float add = nrmS[rl];
#pragma unroll
                    for (int i = 0; i < 16; i++)
                        if (c0 + i < nT) drow[c0 + i] = fmaf(p.alpha, v[i], add);
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        done++;
        if (!ok) {
            if (threadIdx.x == 0) atomicOr(p.flag, 4);
            aborted = true;
        }
        __syncthreads();
        if (aborted) break;
    }
    // ---- teardown: after an abort, let this CTA's own MMAs and copies land
    if (aborted && threadIdx.x == 0) {
        if (mmaPending) {
            umma_commit(drain);     // arrives once every earlier MMA has completed
            mbar_wait(drain, 0, kWaitBudget / 4);
        }
        for (int s = 0; s < S; s++) {
            // the latest B copy into each stage was issued for one of the last S blocks
            for (uint32_t gg = (g >= (uint32_t)S ? g - S : 0); gg < g + S; gg++)
                if ((int)(gg % S) == s) mbar_wait(bFull + s, (gg / S) & 1, kWaitBudget / 16);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(p.tmemCols)
                     : "memory");
    }
}

// Per-particle descriptors of a uniform batch: particle l has nR rotations
// (rows l nR ..), nT translations (rows l nT ..), K pixels and class cls[l]
// (class 0 without cls); its likelihoods are D[l nR nT ..].
__global__ void k_fused_uniform(int nP, int nR, int nT, int K, const int* __restrict__ cls,
                                FusedParticle* __restrict__ part, int* __restrict__ itemOff)
{
    const int items = (nR + FU_M - 1) / FU_M;
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l <= nP; l += gridDim.x * blockDim.x) {
        itemOff[l] = l * items;
        if (l == nP) continue;
        FusedParticle q;
        q.cls = cls ? cls[l] : 0;
        q.nR = nR;
        q.nT = nT;
        q.rowOff = l * nR;
        q.transRow = l * nT;
        q.sgOff = l * K;
        q.dOff = (long long)l * nR * nT;
        part[l] = q;
    }
}

}  // namespace

int fused_items(int nR) { return (nR + FU_M - 1) / FU_M; }

size_t fused_smem_bytes(int vdim, int ntile, int* stagesOut)
{
    const size_t stageBytes = 2 * (size_t)FU_M * FU_BK * 2 + 2 * (size_t)ntile * FU_BK * 2;
    const size_t tail = sizeof(int) * ((size_t)vdim / 2 + 1 + 2 * (size_t)vdim) +
                        sizeof(float) * (FU_M * 9 + FU_M + FU_ROWS * FU_WARPS * 16) + 8 +
                        16 * sizeof(uint64_t) + 12 * sizeof(int) + 16 + sizeof(ItemDesc);
    const size_t limit = 227 * 1024;
    for (int S = 3; S >= 2; S--) {
        const size_t total = 1024 + S * stageBytes + tail;
        if (total <= limit) {
            if (stagesOut) *stagesOut = S;
            return total;
        }
    }
    if (stagesOut) *stagesOut = 0;
    return 0;
}

cudaError_t launch_fused_uniform_setup(int nP, int nR, int nT, int K, const int* cls,
                                       FusedParticle* part, int* itemOff, cudaStream_t st)
{
    k_fused_uniform<<<(nP + 256) / 256, 256, 0, st>>>(nP, nR, nT, K, cls, part,
                                                                     itemOff);
    return cudaGetLastError();
}

cudaError_t launch_fused_bf16x3(float4* const* volTable, int vdim, int pf, const float* mf,
                                const FusedParticle* part, const int* itemOff, int nP,
                                int nItems, const FusedPixels* pix, const float* sigRcp,
                                const float* ctf, const void* B, long long rowsB, int KpB,
                                int maxNT, float* D, float alpha, int* flag, int* counter,
                                cudaStream_t st)
{
    if (nItems <= 0) return cudaSuccess;
    if (maxNT <= 0 || maxNT > 256 || KpB % FU_BK || !tc::encode_fn()) return cudaErrorInvalidValue;
    FusedParams p;
    p.volTable = volTable;
    p.vdim = vdim;
    p.pf = pf;
    p.mf = mf;
    p.part = part;
    p.itemOff = itemOff;
    p.nP = nP;
    p.nItems = nItems;
    for (int c = 0; c < kMaxClasses; c++) p.pix[c] = pix[c];
    p.sigRcp = sigRcp;
    p.ctf = ctf;
    p.D = D;
    p.alpha = alpha;
    p.ntile = (maxNT + 15) / 16 * 16;
    p.tmemCols = 32;
    while (p.tmemCols < p.ntile) p.tmemCols <<= 1;
    p.flag = flag;
    p.counter = counter;
    int S = 0;
    const size_t smem = fused_smem_bytes(vdim, p.ntile, &S);
    if (!smem) return cudaErrorInvalidValue;
    p.stages = S;
    const __nv_bfloat16* Bh = reinterpret_cast<const __nv_bfloat16*>(B);
    const __nv_bfloat16* Bl = Bh + rowsB * KpB;
    CUtensorMap mBh, mBl;
    if (!tc::make_map(&mBh, Bh, rowsB, KpB, p.ntile, FU_BK, true) ||
        !tc::make_map(&mBl, Bl, rowsB, KpB, p.ntile, FU_BK, true))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_fused_bf16x3,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(counter, 0, sizeof(int), st)) != cudaSuccess) return e;
    const int grid = nItems < sms ? nItems : sms;
    k_fused_bf16x3<<<grid, FU_THREADS, smem, st>>>(mBh, mBl, p);
    return cudaGetLastError();
}

}  // namespace tg3
