// tg3_bank_gemm.cu -- the rescoring cross term with the proposals' slices
// read straight from the projection banks.
//
// The learned E-step scores nR proposed rotations x nT translations of every
// particle.  The rotations are rows of its class's projection bank (the
// class projected once at a fixed rotation set), so the slices need no
// projection -- and no copy either: this kernel loads each 128-row A tile of
// the cross-term GEMM from the bank rows the particle proposed, with TMA
// tile::gather4 loads (four rows of one K block per instruction, box one row
// high, 128-byte swizzle), and computes the rows' norms sum_p sigRcp ctf^2
// |P|^2 from the same staged tiles.  Against the gather-then-GEMM form it
// saves, per proposed row, the copy written and read back (8 Kp bytes) and
// the |P|^2 row read for the norm (4 K bytes).
//
// C[l][r][t] = alpha sum_k Ph[l,r][k] (Bh + Bl)[l,t][k] + Pl Bh + nrm[l][r],
// the split-bf16 product of tg3_tc.cu (hi x hi + hi x lo + lo x hi, FP32
// accumulation in tensor memory).  One CTA per (128-row tile, particle),
// 192 threads, warp-specialised:
//   warp 4      : TMA producer (lane 0: the B tiles and the stage's byte
//                 count; every lane: two gather4 loads of the A planes);
//   warp 5      : tensor-memory allocation; lane 0 issues the tcgen05.mma
//                 and commits each stage to its empty barrier;
//   warps 0 - 3 : thread t sums row t's norm in compensated (Kahan) FP32 as
//                 each stage lands, then releases the stage; afterwards the
//                 epilogue (tcgen05.ld 32x32b, + norm, coalesced stores).
// A stage is free when the MMAs that read it have completed and the four
// norm warps have read it (empty barrier count 5).  Every wait is bounded
// (clock budget); on expiry the CTA records TG3 flag bit 4, stops issuing,
// waits (bounded) for its own copies and MMAs, frees its tensor memory and
// returns.  A bank row index outside the particle's bank sets flag bit 16
// and row 0 is read in its place.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg3_internal.cuh"
#include "tg3_tcgen05.cuh"

namespace tg3 {

namespace {

using namespace tc;

constexpr int BG_M = 128;          // rows of A per CTA (UMMA M)
constexpr int BG_BK = 64;          // bf16 elements per K block (one 128-byte row)
constexpr int BG_THREADS = 192;

struct BankMaps {
    CUtensorMap hi[kMaxClasses];
    CUtensorMap lo[kMaxClasses];
    int nB[kMaxClasses];           // rows of each class's bank (0: none)
};

struct BgParams {
    int nR, nT, Kd, K;             // rows / columns per particle, K (bf16 elements), pixels
    int ntile, tmemCols, stages;
    const int* idx;                // [nP][nR] bank rows
    const int* cls;                // [nP] (null: class 0)
    const int* order;              // [nP] particle of each grid row (null: identity)
    const float* sigRcp;           // [nP][K]
    const float* ctf;              // [nP][K]
    float* C;                      // [nP][nR][nT]
    float alpha;
    int* flag;
};

__device__ __forceinline__ void tma_gather4(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int col, int r0, int r1, int r2, int r3)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(col), "r"(r0), "r"(r1), "r"(r2), "r"(r3),
        "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Kahan summation step: s + v with the lost low part kept in c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v)
{
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

__global__ void __launch_bounds__(BG_THREADS, 1)
k_gemm_bank_bf16x3(const __grid_constant__ BankMaps maps, const __grid_constant__ CUtensorMap tmBh,
                   const __grid_constant__ CUtensorMap tmBl, const BgParams p)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int aBytes = BG_M * BG_BK * 2;                  // 16 KB per plane
    const int bBytes = p.ntile * BG_BK * 2;
    const int stageBytes = 2 * aBytes + 2 * bBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + p.stages * stageBytes);
    uint64_t* empty = full + p.stages;
    uint64_t* accum = empty + p.stages;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(accum + 1);
    int* abortFlag = reinterpret_cast<int*>(tmemSlot + 1);
    int* rows = abortFlag + 1;                            // [BG_M] bank rows of the tile

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mtile = blockIdx.x, item = p.order ? p.order[blockIdx.y] : blockIdx.y;
    const int cl = p.cls ? p.cls[item] : 0;
    const bool clOk = cl >= 0 && cl < kMaxClasses && maps.nB[cl] > 0;
    const int k = clOk ? cl : 0;
    const int nB = clOk ? maps.nB[k] : 0;
    const int nkb = p.Kd / BG_BK;
    const int bRow0 = item * p.nT;

    if (threadIdx.x < BG_M) {
        const int r = mtile * BG_M + threadIdx.x;
        int b = 0;
        if (r < p.nR) {
            b = p.idx[(size_t)item * p.nR + r];
            if (b < 0 || b >= nB) {
                atomicOr(p.flag, 1 << 16);
                b = 0;
            }
        }
        rows[threadIdx.x] = b;
    }
    if (threadIdx.x == BG_M) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 5);
        }
        mbar_init(accum, 1);
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 5) {
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

    int issuedTma = 0;      // K blocks whose copies were issued (producer lane 0)
    int issuedMma = 0;      // K blocks whose MMAs were issued (issuer)
    float nrmS = 0.f, nrmC = 0.f;
    if (warp == 4) {
        // ---------------- TMA producer
        const CUtensorMap* mh = &maps.hi[k];
        const CUtensorMap* ml = &maps.lo[k];
        const int r0 = rows[4 * lane], r1 = rows[4 * lane + 1], r2 = rows[4 * lane + 2],
                  r3 = rows[4 * lane + 3];
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % p.stages;
            const int round = kb / p.stages;
            int go = 1;
            uint8_t* st = smem + s * stageBytes;
            if (lane == 0) {
                if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1, kWaitBudget)) {
                    atomicOr(p.flag, 4);
                    *(volatile int*)abortFlag = 1;
                    go = 0;
                } else if (*(volatile int*)abortFlag) {
                    go = 0;
                } else {
                    mbar_expect_tx(full + s, stageBytes);
                    tma_load_2d(st + 2 * aBytes, &tmBh, full + s, kb * BG_BK, bRow0);
                    tma_load_2d(st + 2 * aBytes + bBytes, &tmBl, full + s, kb * BG_BK, bRow0);
                    issuedTma = kb + 1;
                }
            }
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) break;
            // rows 4 lane .. 4 lane + 3 of both planes: 512 bytes each
            tma_gather4(st + lane * 512, mh, full + s, kb * BG_BK, r0, r1, r2, r3);
            tma_gather4(st + aBytes + lane * 512, ml, full + s, kb * BG_BK, r0, r1, r2, r3);
        }
    } else if (warp == 5) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = umma_idesc(BG_M, p.ntile);
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % p.stages;
                const int round = kb / p.stages;
                if (!mbar_wait(full + s, round & 1, kWaitBudget)) {
                    atomicOr(p.flag, 4);
                    *(volatile int*)abortFlag = 1;
                    break;
                }
                if (*(volatile int*)abortFlag) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                uint8_t* st = smem + s * stageBytes;
                const uint32_t ah = smem_u32(st), al = smem_u32(st + aBytes);
                const uint32_t bh = smem_u32(st + 2 * aBytes),
                               bl = smem_u32(st + 2 * aBytes + bBytes);
#pragma unroll
                for (int kk = 0; kk < BG_BK / 16; kk++) {
                    const uint32_t off = kk * 32;
                    umma_bf16(tmem, umma_desc(ah + off), umma_desc(bh + off), idesc,
                              (kb | kk) != 0);
                    umma_bf16(tmem, umma_desc(ah + off), umma_desc(bl + off), idesc, 1);
                    umma_bf16(tmem, umma_desc(al + off), umma_desc(bh + off), idesc, 1);
                }
                umma_commit(empty + s);
                issuedMma = kb + 1;
            }
            umma_commit(accum);
        }
    } else {
        // ---------------- norm of row t = threadIdx.x, stage by stage
        const int t = threadIdx.x;
        const float* sg = p.sigRcp + (size_t)item * p.K;
        const float* cf = p.ctf + (size_t)item * p.K;
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % p.stages;
            const int round = kb / p.stages;
            if (!mbar_wait(full + s, round & 1, kWaitBudget)) {
                atomicOr(p.flag, 4);
                *(volatile int*)abortFlag = 1;
                break;
            }
            const uint8_t* st = smem + s * stageBytes;
            const uint8_t* rh = st + t * 128;
            const uint8_t* rl = st + aBytes + t * 128;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                // logical 16-byte chunk j of the row sits at chunk j ^ (row % 8)
                const int ph = ((j ^ (t & 7)) << 4);
                const uint4 h = *reinterpret_cast<const uint4*>(rh + ph);
                const uint4 lo = *reinterpret_cast<const uint4*>(rl + ph);
                const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {lo.x, lo.y, lo.z, lo.w};
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int px = kb * (BG_BK / 2) + j * 4 + q;
                    if (px < p.K) {
                        const float2 hf = __bfloat1622float2(
                            *reinterpret_cast<const __nv_bfloat162*>(&hw[q]));
                        const float2 lf = __bfloat1622float2(
                            *reinterpret_cast<const __nv_bfloat162*>(&lw[q]));
                        const float re = hf.x + lf.x, im = hf.y + lf.y;
                        const float c = __ldg(cf + px);
                        kahan_add(nrmS, nrmC, __ldg(sg + px) * c * c * (re * re + im * im));
                    }
                }
            }
            // generic reads of this stage done before the producer's next
            // asynchronous copy into it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + s);
        }
    }
    __syncthreads();
    // ---------------- epilogue (warps 0 - 3)
    bool ok = *(volatile int*)abortFlag == 0;
    if (warp < 4) ok = ok && mbar_wait(accum, 0, kWaitBudget);
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) {
        atomicOr(p.flag, 4);
        *(volatile int*)abortFlag = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool aborted = !ok;
    if (!aborted && warp < 4) {
        const int pitch = p.ntile + 1;
        float* stage = reinterpret_cast<float*>(smem) + (size_t)warp * 32 * pitch;
        const int rowBase = mtile * BG_M + warp * 32;
        const float add = nrmS - nrmC;
        for (int c0 = 0; c0 < p.ntile; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) stage[lane * pitch + c0 + i] = fmaf(p.alpha, v[i], add);
        }
        __syncwarp();
        float* cbase = p.C + (size_t)item * p.nR * p.nT;
        for (int rr = 0; rr < 32; rr++) {
            const int r = rowBase + rr;
            if (r >= p.nR) break;
            for (int j = lane; j < p.nT; j += 32) cbase[(size_t)r * p.nT + j] = stage[rr * pitch + j];
        }
    }
    // on an abort, the copies and MMAs this CTA issued are waited for (bounded)
    if (aborted && warp == 4 && lane == 0) {
        for (int kb = 0; kb < issuedTma; kb++) {
            const int s = kb % p.stages;
            mbar_wait(full + s, (kb / p.stages) & 1, kWaitBudget / 4);
        }
    }
    if (aborted && warp == 5 && lane == 0 && issuedMma > 0) mbar_wait(accum, 0, kWaitBudget / 4);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 5) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(p.tmemCols)
                     : "memory");
    }
}


// The same product with the A tiles gathered by the four norm warps
// themselves with cp.async: per K block every thread copies 16 bytes of each
// plane of 8 rows straight to their swizzled places in shared memory (8
// lanes cover a row's 128-byte chunk, so a warp instruction reads 4 whole
// rows' chunks), with no register staging.  The wait for a K block's copies
// lags their issue by LAG = S - 3 blocks (cp.async.wait_group LAG): the
// copies of LAG + 1 blocks are in flight, and the MMAs of a block have two
// blocks' time to finish before the producers need its stage again (with a
// lag of S - 1 the producers stalled every block on the MMA round trip).
// Once the thread's own copies of a K block have landed it makes them
// visible to the tensor cores (proxy fence), arrives, and then adds their
// |P|^2, weighted by sigRcp ctf^2, to its partial norms (a plain FP32 sum
// of each row's four pixels, added to the running sum in compensated FP32;
// the lanes' partials are summed at the end).  A stage is full when the
// gather warps have arrived and the B tiles' bytes have landed (TMA); it is
// free when the MMAs that read it have completed.
struct LdgRows {
    const __nv_bfloat16* hi[kMaxClasses];
    const __nv_bfloat16* lo[kMaxClasses];
    int nB[kMaxClasses];
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}

// CP_PW gather warps (eight by default, 0 - 7), then the B-tile TMA warp
// (CP_PW) and the MMA warp (CP_PW + 1, which also holds the tensor memory);
// warps 0 - 3 run the epilogue.
//
// BK is the K block: 64 bf16 (128-byte rows, 128-byte swizzle) or 32
// (64-byte rows, 64-byte swizzle: half the bytes a stage, so more stages, or
// two CTAs an SM with MINB = 2).  A row's chunk of a K block is BK / 8
// 16-byte pieces, one per lane of a row group; a thread copies CP_RPT rows.
constexpr int cp_threads(int pw) { return (pw + 2) * 32; }

template <int BK>
__device__ __forceinline__ uint64_t bank_desc(uint32_t saddr)
{
    return BK == 64 ? umma_desc(saddr) : umma_desc_sw64(saddr);
}

// Byte offset of 16-byte chunk q of row r of an A plane: 128-byte rows with
// the 128-byte swizzle (chunk XOR row mod 8) or 64-byte rows with the
// 64-byte swizzle (8-row groups of 512 bytes, chunk XOR (row / 2) mod 4).
template <int BK>
__device__ __forceinline__ int bank_phys(int r, int q)
{
    return BK == 64 ? r * 128 + ((q ^ (r & 7)) << 4)
                    : (r >> 3) * 512 + (r & 7) * 64 + ((q ^ ((r >> 1) & 3)) << 4);
}

template <int S, int BK, int MINB, int CP_PW = 8>
__global__ void __launch_bounds__(cp_threads(CP_PW), MINB)
k_gemm_bank_cp(const LdgRows banks, const __grid_constant__ CUtensorMap tmBh,
               const __grid_constant__ CUtensorMap tmBl, const BgParams p)
{
    constexpr int QPR = BK / 8;                          // 16-byte chunks per row
    constexpr int CP_RPT = BG_M * QPR / (CP_PW * 32);     // rows per gather thread
    constexpr int RSTRIDE = CP_PW * 32 / QPR;             // rows between a thread's rows
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int aBytes = BG_M * BK * 2;
    const int bBytes = p.ntile * BK * 2;
    const int stageBytes = 2 * aBytes + 2 * bBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + S * stageBytes);
    uint64_t* empty = full + S;
    uint64_t* accum = empty + S;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(accum + 1);
    int* abortFlag = reinterpret_cast<int*>(tmemSlot + 1);
    int* rows = abortFlag + 1;                            // [BG_M]
    float* nrmRow = reinterpret_cast<float*>(rows + BG_M);  // [BG_M]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mtile = blockIdx.x, item = p.order ? p.order[blockIdx.y] : blockIdx.y;
    const int cl = p.cls ? p.cls[item] : 0;
    const bool clOk = cl >= 0 && cl < kMaxClasses && banks.nB[cl] > 0;
    const int k = clOk ? cl : 0;
    const int nB = clOk ? banks.nB[k] : 0;
    const int nkb = p.Kd / BK;
    const int bRow0 = item * p.nT;

    if (threadIdx.x < BG_M) {
        const int r = mtile * BG_M + threadIdx.x;
        int b = 0;
        if (r < p.nR) {
            b = p.idx[(size_t)item * p.nR + r];
            if (b < 0 || b >= nB) {
                atomicOr(p.flag, 1 << 16);
                b = 0;
            }
        }
        rows[threadIdx.x] = b;
    }
    if (threadIdx.x == BG_M) {
        for (int s = 0; s < S; s++) {
            mbar_init(full + s, CP_PW + 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accum, 1);
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == CP_PW + 1) {
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

    int issuedTma = 0, issuedMma = 0;
    if (warp < CP_PW) {
        // ---------------- A tiles and the rows' norms
        const int t = threadIdx.x;
        const int g = t / QPR, q = t % QPR;                // row group, 16-byte chunk
        const __nv_bfloat16* bh = banks.hi[k];
        const __nv_bfloat16* bl = banks.lo[k];
        const __nv_bfloat16* srcH[CP_RPT];
        const __nv_bfloat16* srcL[CP_RPT];
        int phys[CP_RPT];
#pragma unroll
        for (int i = 0; i < CP_RPT; i++) {
            const int r = g + RSTRIDE * i;
            const size_t off = (size_t)rows[r] * p.Kd + q * 8;
            srcH[i] = bh + off;
            srcL[i] = bl + off;
            phys[i] = bank_phys<BK>(r, q);
        }
        const float* sg = p.sigRcp + (size_t)item * p.K;
        const float* cf = p.ctf + (size_t)item * p.K;
        float nS[CP_RPT], nC[CP_RPT];
#pragma unroll
        for (int i = 0; i < CP_RPT; i++) nS[i] = nC[i] = 0.f;
        // the weights sigRcp ctf^2 of this lane's 4 pixels, one K block ahead
        auto weights = [&](int kd, float* w) {
            const int px0 = kd * (BK / 2) + q * 4;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int px = px0 + c;
                const float cc = px < p.K ? __ldg(cf + px) : 0.f;
                w[c] = px < p.K ? __ldg(sg + px) * cc * cc : 0.f;
            }
        };
        float wCur[4], wNext[4];
        weights(0, wCur);
        constexpr int LAG = S > 3 ? S - 3 : 0;
        for (int kb = 0; kb < nkb + LAG; kb++) {
            if (kb < nkb) {
                const int s = kb % S;
                const int round = kb / S;
                if (round > 0) {
                    bool ok = lane != 0 || mbar_wait(empty + s, (round - 1) & 1, kWaitBudget);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok || *(volatile int*)abortFlag) {
                        if (lane == 0) {
                            atomicOr(p.flag, 4);
                            *(volatile int*)abortFlag = 1;
                        }
                        break;
                    }
                }
                uint8_t* st = smem + s * stageBytes;
                const size_t o = (size_t)kb * BK;
#pragma unroll
                for (int i = 0; i < CP_RPT; i++) {
                    cp_async16(st + phys[i], srcH[i] + o);
                    cp_async16(st + aBytes + phys[i], srcL[i] + o);
                }
            }
            // one group per iteration (empty at the tail), so that
            // "LAG groups pending" always means K block kb - LAG landed
            asm volatile("cp.async.commit_group;" ::: "memory");
            const int kd = kb - LAG;
            if (kd < 0) continue;
            if (kd + 1 < nkb) weights(kd + 1, wNext);
            asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
            // the copies (generic proxy) visible to the tensor cores' reads;
            // the stage is handed over before this thread's norm reads of it
            // (reads both, and only this thread rewrites its chunks, S blocks on)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(full + kd % S);
            const uint8_t* st = smem + (kd % S) * stageBytes;
#pragma unroll
            for (int i = 0; i < CP_RPT; i++) {
                const uint4 h = *reinterpret_cast<const uint4*>(st + phys[i]);
                const uint4 lo = *reinterpret_cast<const uint4*>(st + aBytes + phys[i]);
                const uint32_t hw[4] = {h.x, h.y, h.z, h.w}, lw[4] = {lo.x, lo.y, lo.z, lo.w};
                float part = 0.f;
#pragma unroll
                for (int c = 0; c < 4; c++) {
                    const float2 hf = __bfloat1622float2(
                        *reinterpret_cast<const __nv_bfloat162*>(&hw[c]));
                    const float2 lf = __bfloat1622float2(
                        *reinterpret_cast<const __nv_bfloat162*>(&lw[c]));
                    const float re = hf.x + lf.x, im = hf.y + lf.y;
                    part = fmaf(wCur[c], re * re + im * im, part);
                }
                kahan_add(nS[i], nC[i], part);
            }
#pragma unroll
            for (int c = 0; c < 4; c++) wCur[c] = wNext[c];
        }
        // copies still in flight after an abort land before the CTA leaves
        asm volatile("cp.async.wait_all;" ::: "memory");
        // the rows' norms: the QPR lanes of a row group hold partials
#pragma unroll
        for (int i = 0; i < CP_RPT; i++) {
            float v = nS[i] - nC[i];
#pragma unroll
            for (int o = 1; o < QPR; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (q == 0) nrmRow[g + RSTRIDE * i] = v;
        }
    } else if (warp == CP_PW) {
        // ---------------- B tiles (TMA)
        if (lane == 0) {
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % S;
                const int round = kb / S;
                if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1, kWaitBudget)) {
                    atomicOr(p.flag, 4);
                    *(volatile int*)abortFlag = 1;
                    break;
                }
                if (*(volatile int*)abortFlag) break;
                uint8_t* st = smem + s * stageBytes;
                mbar_expect_tx(full + s, 2 * bBytes);
                tma_load_2d(st + 2 * aBytes, &tmBh, full + s, kb * BK, bRow0);
                tma_load_2d(st + 2 * aBytes + bBytes, &tmBl, full + s, kb * BK, bRow0);
                issuedTma = kb + 1;
            }
        }
    } else {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = umma_idesc(BG_M, p.ntile);
            for (int kb = 0; kb < nkb; kb++) {
                const int s = kb % S;
                const int round = kb / S;
                if (!mbar_wait(full + s, round & 1, kWaitBudget)) {
                    atomicOr(p.flag, 4);
                    *(volatile int*)abortFlag = 1;
                    break;
                }
                if (*(volatile int*)abortFlag) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                uint8_t* st = smem + s * stageBytes;
                const uint32_t ah = smem_u32(st), al = smem_u32(st + aBytes);
                const uint32_t bh = smem_u32(st + 2 * aBytes),
                               bl = smem_u32(st + 2 * aBytes + bBytes);
#pragma unroll
                for (int kk = 0; kk < BK / 16; kk++) {
                    const uint32_t off = kk * 32;
                    umma_bf16(tmem, bank_desc<BK>(ah + off), bank_desc<BK>(bh + off), idesc,
                              (kb | kk) != 0);
                    umma_bf16(tmem, bank_desc<BK>(ah + off), bank_desc<BK>(bl + off), idesc, 1);
                    umma_bf16(tmem, bank_desc<BK>(al + off), bank_desc<BK>(bh + off), idesc, 1);
                }
                umma_commit(empty + s);
                issuedMma = kb + 1;
            }
            umma_commit(accum);
        }
    }
    __syncthreads();
    // ---------------- epilogue (warps 0 - 3)
    bool ok = *(volatile int*)abortFlag == 0;
    if (warp < 4) ok = ok && mbar_wait(accum, 0, kWaitBudget);
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) {
        atomicOr(p.flag, 4);
        *(volatile int*)abortFlag = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool aborted = !ok;
    if (!aborted && warp < 4) {
        const int pitch = p.ntile + 1;
        float* stage = reinterpret_cast<float*>(smem) + (size_t)warp * 32 * pitch;
        const int rowBase = mtile * BG_M + warp * 32;
        const float add = nrmRow[warp * 32 + lane];
        for (int c0 = 0; c0 < p.ntile; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) stage[lane * pitch + c0 + i] = fmaf(p.alpha, v[i], add);
        }
        __syncwarp();
        float* cbase = p.C + (size_t)item * p.nR * p.nT;
        for (int rr = 0; rr < 32; rr++) {
            const int r = rowBase + rr;
            if (r >= p.nR) break;
            for (int j = lane; j < p.nT; j += 32) cbase[(size_t)r * p.nT + j] = stage[rr * pitch + j];
        }
    }
    if (aborted && warp == CP_PW && lane == 0) {
        for (int kb = 0; kb < issuedTma; kb++) {
            const int s = kb % S;
            mbar_wait(full + s, (kb / S) & 1, kWaitBudget / 4);
        }
    }
    if (aborted && warp == CP_PW + 1 && lane == 0 && issuedMma > 0)
        mbar_wait(accum, 0, kWaitBudget / 4);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == CP_PW + 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(p.tmemCols)
                     : "memory");
    }
}

// The visiting order of the particles: sorted by (class, first proposed bank
// row), ties by particle index; one CTA, bitonic sort of n <= 8192 keys in
// shared memory.  A row outside [0, 2^24) or a class outside [0, 2^7) only
// moves its particle.
__global__ void k_bank_order(const int* __restrict__ idx, const int* __restrict__ cls, int nP,
                             int nR, int nPow2, int* __restrict__ order)
{
    extern __shared__ unsigned long long key[];
    for (int l = threadIdx.x; l < nPow2; l += blockDim.x) {
        unsigned long long v = ~0ull;
        if (l < nP) {
            const unsigned r = (unsigned)idx[(size_t)l * nR] & 0xffffffu;
            const unsigned c = cls ? (unsigned)cls[l] & 0x7fu : 0u;
            v = ((unsigned long long)((c << 24) | r) << 32) | (unsigned)l;
        }
        key[l] = v;
    }
    __syncthreads();
    for (int size = 2; size <= nPow2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < nPow2 / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const unsigned long long a = key[lo], b = key[hi];
                if ((a > b) == asc) {
                    key[lo] = b;
                    key[hi] = a;
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < nP; i += blockDim.x) order[i] = (int)(key[i] & 0xffffffffu);
}

}  // namespace

// A: the classes' banks (bank[k].hi holds the hi plane, then the lo plane
// nB Kd elements later); B: the shifted data, hi plane [nP nT][Kd] then the
// lo plane.  C [nP][nR][nT] = alpha (split product) + the rows' norms.
cudaError_t launch_gemm_bank_bf16x3(const Bank* banks, unsigned pixGen, const int* idx,
                                    const int* cls, int nP, int nR, const void* B, int nT,
                                    int Kd, int K, const float* sigRcp, const float* ctf,
                                    float* C, float alpha, int* flag, cudaStream_t st,
                                    bool tmaGather, int* order, int shape)
{
    if (shape < 0 || shape > 3) return cudaErrorInvalidValue;
    if (nP <= 0 || nR <= 0 || nT <= 0 || nT > 256 || Kd <= 0 || Kd % BG_BK || nP > 65535)
        return cudaErrorInvalidValue;
    BankMaps maps;
    int first = -1;
    for (int k = 0; k < kMaxClasses; k++) {
        const Bank& b = banks[k];
        const bool ok = b.nB > 0 && b.gen == pixGen && b.Kp == Kd;
        maps.nB[k] = ok ? b.nB : 0;
        if (ok && first < 0) first = k;
    }
    if (first < 0) return cudaErrorInvalidValue;
    for (int k = 0; k < kMaxClasses; k++) {
        const Bank& b = banks[maps.nB[k] ? k : first];
        const __nv_bfloat16* hi = b.hi;
        const __nv_bfloat16* lo = b.hi + (size_t)b.nB * b.Kp;
        // one-row boxes: the rows of a tile are gathered four at a time
        if (!tc::make_map(&maps.hi[k], hi, b.nB, Kd, 1) || !tc::make_map(&maps.lo[k], lo, b.nB, Kd, 1))
            return cudaErrorInvalidValue;
    }
    BgParams p;
    p.nR = nR;
    p.nT = nT;
    p.Kd = Kd;
    p.K = K;
    p.ntile = (nT + 15) / 16 * 16;
    p.tmemCols = 32;
    while (p.tmemCols < p.ntile) p.tmemCols <<= 1;
    const int stageBytes = 2 * BG_M * BG_BK * 2 + 2 * p.ntile * BG_BK * 2;
    p.stages = (200 * 1024) / stageBytes;
    if (p.stages > 4) p.stages = 4;
    if (p.stages < 2) return cudaErrorInvalidValue;
    if ((size_t)BG_M * (p.ntile + 1) * 4 > (size_t)p.stages * stageBytes)
        return cudaErrorInvalidValue;
    p.idx = idx;
    p.cls = cls;
    p.order = nullptr;
    if (order && nP <= 8192) {
        int n2 = 1;
        while (n2 < nP) n2 <<= 1;
        const size_t sm = sizeof(unsigned long long) * n2;
        if (sm > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(k_bank_order,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)sm);
            if (e != cudaSuccess) return e;
        }
        k_bank_order<<<1, 1024, sm, st>>>(idx, cls, nP, nR, n2, order);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        p.order = order;
    }
    p.sigRcp = sigRcp;
    p.ctf = ctf;
    p.C = C;
    p.alpha = alpha;
    p.flag = flag;
    const __nv_bfloat16* Bh = reinterpret_cast<const __nv_bfloat16*>(B);
    const __nv_bfloat16* Bl = Bh + (size_t)nP * nT * Kd;
    CUtensorMap mBh, mBl;
    if (!tc::make_map(&mBh, Bh, (long long)nP * nT, Kd, p.ntile) ||
        !tc::make_map(&mBl, Bl, (long long)nP * nT, Kd, p.ntile))
        return cudaErrorInvalidValue;
    // stages, then barriers (2 stages + 1, 8 bytes each), the TMEM slot, the
    // abort word and the tile's row list
    const size_t smem = 1024 + (size_t)p.stages * stageBytes + 256 + 2 * sizeof(int) * BG_M;
    dim3 grid((nR + BG_M - 1) / BG_M, nP);
    if (tmaGather) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_bank_bf16x3,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_bank_bf16x3<<<grid, BG_THREADS, smem, st>>>(maps, mBh, mBl, p);
        return cudaGetLastError();
    }
    LdgRows rowsOf;
    for (int k = 0; k < kMaxClasses; k++) {
        const Bank& b = banks[maps.nB[k] ? k : first];
        rowsOf.hi[k] = b.hi;
        rowsOf.lo[k] = b.hi + (size_t)b.nB * b.Kp;
        rowsOf.nB[k] = maps.nB[k];
    }
    // the cp.async form keeps every stage in flight: as many as fit in one
    // CTA's (shape 0: K blocks of 64, <= 5 stages; shape 1: of 32, <= 9) or
    // in half an SM's shared memory (shape 2: K blocks of 32, two CTAs an SM)
    using KernFn = void (*)(const LdgRows, const CUtensorMap, const CUtensorMap, const BgParams);
    const int bk = shape == 0 || shape == 3 ? 64 : 32;
    const int stageCp = 2 * BG_M * bk * 2 + 2 * p.ntile * bk * 2;
    const size_t fixed = 1024 + 256 + 2 * sizeof(int) * BG_M;
    const size_t budget = shape == 2 ? 113 * 1024 : 227 * 1024;
    int S = (int)((budget - fixed) / stageCp);
    const int maxS = shape == 0 || shape == 3 ? 5 : shape == 1 ? 9 : 4;
    if (S > maxS) S = maxS;
    if (S < 2 || (size_t)BG_M * (p.ntile + 1) * 4 > (size_t)S * stageCp)
        return cudaErrorInvalidValue;
    KernFn kern = nullptr;
    if (shape == 0)
        kern = S == 5 ? k_gemm_bank_cp<5, 64, 1> : S == 4 ? k_gemm_bank_cp<4, 64, 1>
             : S == 3 ? k_gemm_bank_cp<3, 64, 1> : k_gemm_bank_cp<2, 64, 1>;
    else if (shape == 3)
        kern = S == 5 ? k_gemm_bank_cp<5, 64, 1, 16> : S == 4 ? k_gemm_bank_cp<4, 64, 1, 16>
             : S == 3 ? k_gemm_bank_cp<3, 64, 1, 16> : k_gemm_bank_cp<2, 64, 1, 16>;
    else if (shape == 1) {
        S = S >= 9 ? 9 : S >= 8 ? 8 : S >= 6 ? 6 : S >= 4 ? 4 : 2;   // the instantiated depths
        kern = S == 9 ? k_gemm_bank_cp<9, 32, 1> : S == 8 ? k_gemm_bank_cp<8, 32, 1>
             : S == 6 ? k_gemm_bank_cp<6, 32, 1> : S == 4 ? k_gemm_bank_cp<4, 32, 1>
                                                : k_gemm_bank_cp<2, 32, 1>;
    } else
        kern = S == 4 ? k_gemm_bank_cp<4, 32, 2> : S == 3 ? k_gemm_bank_cp<3, 32, 2>
                                                         : k_gemm_bank_cp<2, 32, 2>;
    p.stages = S;
    CUtensorMap cBh = mBh, cBl = mBl;
    if (bk == 32 && (!tc::make_map(&cBh, Bh, (long long)nP * nT, Kd, p.ntile, 32, true) ||
                     !tc::make_map(&cBl, Bl, (long long)nP * nT, Kd, p.ntile, 32, true)))
        return cudaErrorInvalidValue;
    const size_t smemCp = fixed + (size_t)S * stageCp;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smemCp);
    if (e != cudaSuccess) return e;
    kern<<<grid, cp_threads(shape == 3 ? 16 : 8), smemCp, st>>>(rowsOf, cBh, cBl, p);
    return cudaGetLastError();
}

}  // namespace tg3
