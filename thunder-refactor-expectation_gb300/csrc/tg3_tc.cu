// tg3_tc.cu -- the likelihood cross term on the 5th-generation tensor cores.
//
// C[b][i][j] = alpha * sum_k A[b][i][k] B[b][j][k] + nrm[b][i], with each FP32
// operand stored as two bf16 planes, hi = bf16(x) and lo = bf16(x - hi), and
// the product formed as Ah Bh + Ah Bl + Al Bh (the lo x lo term, ~2^-16 of
// the product, is dropped), accumulated in FP32 in tensor memory.
//
// One CTA per (128-row tile of A, batch item); N (<= 256) columns in one
// UMMA of shape 128 x N x 16.  128 threads:
//   warp 0 lane 0 : TMA producer (cp.async.bulk.tensor, 128B swizzle),
//   warp 1 lane 0 : tcgen05.mma issuer, commits to the stage's empty barrier,
//   warps 0-3     : epilogue (tcgen05.ld 32x32b, + nrm, store).
// Every mbarrier wait is bounded (clock64 budget); on expiry the CTA records
// TG3 flag bit 4, stops issuing, waits (bounded) for its own copies and MMAs,
// frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg3_internal.cuh"
#include "tg3_tcgen05.cuh"

namespace tg3 {

namespace {

using namespace tc;

constexpr int TC_M = 128;          // rows of A per CTA (UMMA M)
constexpr int TC_BK = 64;          // bf16 elements per K block (one 128-byte row)
constexpr int TC_THREADS = 128;
struct TcParams {
    int M, N, Kd;            // rows of A per item, columns (rows of B) per item, K
    int aRowsPerItem;        // A row offset between items (0: A shared by all items)
    int bRowsPerItem;        // B row offset between items
    int nTotal;              // > 0: columns of the whole problem (the last item is partial)
    int colPerItem;          // column offset between items (column-group remap)
    int cGroup;              // > 0: column j goes to group j / cGroup, position j % cGroup
    long long cGroupStride;  // element stride between column groups
    int ntile;               // N rounded up to 16 (the UMMA N)
    int tmemCols;            // power of two >= ntile
    int stages;
    float* C;
    long long sC;
    int ldc;
    const float* nrm;
    long long sN;
    float alpha;
    int* flag;
};

// K-major operand descriptors: 128-byte rows with the 128-byte swizzle
// (K blocks of 64 bf16) or 64-byte rows with the 64-byte swizzle (K blocks
// of 32, half the stage bytes and so twice the stages in flight).
template <int BK>
__device__ __forceinline__ uint64_t desc(uint32_t saddr)
{
    return BK == 64 ? umma_desc(saddr) : umma_desc_sw64(saddr);
}

template <int BK>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_bf16x3(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
              const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
              const TcParams p)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte aligned stage buffers
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int aBytes = TC_M * BK * 2;                  // 16 KB (BK 64) or 8 KB (32)
    const int bBytes = p.ntile * BK * 2;               // ntile rows of 2 BK bytes
    const int stageBytes = 2 * aBytes + 2 * bBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + p.stages * stageBytes);
    uint64_t* empty = full + p.stages;
    uint64_t* accum = empty + p.stages;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(accum + 1);
    int* abortFlag = reinterpret_cast<int*>(tmemSlot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mtile = blockIdx.x, item = blockIdx.y;
    const int aRow0 = item * p.aRowsPerItem + mtile * TC_M;
    const int bRow0 = item * p.bRowsPerItem;
    const int nValid = p.nTotal > 0 ? min(p.N, p.nTotal - item * p.N) : p.N;
    const int nkb = p.Kd / BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accum, 1);
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
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

    int issuedTma = 0;      // K blocks whose copies were issued (producer)
    int issuedMma = 0;      // K blocks whose MMAs were issued (issuer)
    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % p.stages;
            const int round = kb / p.stages;
            if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1, kWaitBudget)) {
                atomicOr(p.flag, 4);
                *(volatile int*)abortFlag = 1;
                break;
            }
            if (*(volatile int*)abortFlag) break;
            uint8_t* st = smem + s * stageBytes;
            mbar_expect_tx(full + s, stageBytes);
            tma_load_2d(st, &tmAh, full + s, kb * BK, aRow0);
            tma_load_2d(st + aBytes, &tmAl, full + s, kb * BK, aRow0);
            tma_load_2d(st + 2 * aBytes, &tmBh, full + s, kb * BK, bRow0);
            tma_load_2d(st + 2 * aBytes + bBytes, &tmBl, full + s, kb * BK, bRow0);
            issuedTma = kb + 1;
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        const uint32_t idesc = umma_idesc(TC_M, p.ntile);
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
            const uint32_t bh = smem_u32(st + 2 * aBytes), bl = smem_u32(st + 2 * aBytes + bBytes);
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++) {
                const uint32_t off = kk * 32;      // 16 bf16 = 32 bytes along K
                umma_bf16(tmem, desc<BK>(ah + off), desc<BK>(bh + off), idesc,
                          (kb | kk) != 0);
                umma_bf16(tmem, desc<BK>(ah + off), desc<BK>(bl + off), idesc, 1);
                umma_bf16(tmem, desc<BK>(al + off), desc<BK>(bh + off), idesc, 1);
            }
            umma_commit(empty + s);        // stage free once these MMAs have read it
            issuedMma = kb + 1;
        }
        umma_commit(accum);                // all issued MMAs complete -> epilogue
    }
    __syncthreads();
    // ---------------- epilogue (all four warps)
    bool ok = *(volatile int*)abortFlag == 0 && mbar_wait(accum, 0, kWaitBudget);
    // block-uniform decision (the tcgen05.ld below is warp-collective)
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) {
        atomicOr(p.flag, 4);
        *(volatile int*)abortFlag = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool aborted = !ok;
    if (!aborted) {
        // The pipeline stages are free once the accumulator is complete: stage
        // the warp's 32 rows there, then write every row with lanes over
        // columns (coalesced).  Rows are padded by one float so both the
        // column-wise fill and the row-wise drain are free of bank conflicts.
        const int pitch = p.ntile + 1;
        float* stage = reinterpret_cast<float*>(smem) + (size_t)warp * 32 * pitch;
        const int rowBase = mtile * TC_M + warp * 32;
        const bool rowOk = rowBase + lane < p.M;
        const float add = (rowOk && p.nrm) ? p.nrm[item * p.sN + rowBase + lane] : 0.f;
        for (int c0 = 0; c0 < p.ntile; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) stage[lane * pitch + c0 + i] = fmaf(p.alpha, v[i], add);
        }
        __syncwarp();
        float* cbase = p.C + item * p.sC;
        for (int rr = 0; rr < 32; rr++) {
            const int r = rowBase + rr;
            if (r >= p.M) break;
            for (int j = lane; j < nValid; j += 32) {
                size_t off;
                if (p.cGroup > 0) {
                    const int jj = item * p.colPerItem + j;
                    const int l = jj / p.cGroup;
                    off = (size_t)l * p.cGroupStride + (size_t)r * p.ldc + (jj - l * p.cGroup);
                } else {
                    off = (size_t)r * p.ldc + j;
                }
                cbase[off] = stage[rr * pitch + j];
            }
        }
    }
    // on an abort, let the copies this CTA issued land before leaving
    if (aborted && warp == 0 && lane == 0) {
        for (int kb = 0; kb < issuedTma; kb++) {
            const int s = kb % p.stages;
            mbar_wait(full + s, (kb / p.stages) & 1, kWaitBudget / 4);
        }
    }
    // on an abort, the MMA issuer waits (bounded) for the MMAs it issued
    if (aborted && warp == 1 && lane == 0 && issuedMma > 0)
        mbar_wait(accum, 0, kWaitBudget / 4);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(p.tmemCols)
                     : "memory");
    }
}

// ------------------------------------------------------------------------
// The same product for a pair of CTAs on neighbouring row tiles (a cluster of
// two along x) that share their B tile: each CTA loads its own A tile and
// half of the B rows, multicast into both CTAs' shared memory, so each SM
// pulls half of the B bytes from L2.  A stage is full when this CTA's A
// planes and both halves of B have landed (one expect_tx of the whole stage:
// the peer's half signals this CTA's barrier at the same offset); it is free
// when the MMAs of BOTH CTAs that read it have completed (each MMA commit
// arrives on both CTAs' empty barriers, count 2), since a CTA's next copy into
// the stage also writes the peer's copy of it.  The barriers are initialised
// in both CTAs before either issues a copy (cluster barrier), and neither
// leaves before the other has finished (cluster barrier at the end): a
// peer's commit or copy never reaches a CTA that has gone.  Waits are bounded
// as in k_gemm_bf16x3; an expired wait leaves both CTAs to time out and meet
// at the final barrier.
__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d_mc(void* dst, const CUtensorMap* map, uint64_t* bar,
                                               int c0, int c1, uint16_t mask)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        ".multicast::cluster [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar)), "h"(mask)
        : "memory");
}

__device__ __forceinline__ void umma_commit_mc(uint64_t* bar, uint16_t mask)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
        " [%0], %1;" ::"r"(smem_u32(bar)),
        "h"(mask)
        : "memory");
}

template <int BK>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_gemm_bf16x3_pair(const __grid_constant__ CUtensorMap tmAh, const __grid_constant__ CUtensorMap tmAl,
                   const __grid_constant__ CUtensorMap tmBh, const __grid_constant__ CUtensorMap tmBl,
                   const TcParams p)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int aBytes = TC_M * BK * 2;
    const int bBytes = p.ntile * BK * 2;
    const int halfRows = p.ntile / 2;                     // B rows each CTA loads
    const int stageBytes = 2 * aBytes + 2 * bBytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + p.stages * stageBytes);
    uint64_t* empty = full + p.stages;
    uint64_t* accum = empty + p.stages;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(accum + 1);
    int* abortFlag = reinterpret_cast<int*>(tmemSlot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const uint16_t both = 0x3;
    const int mtile = blockIdx.x, item = blockIdx.y;
    const int aRow0 = item * p.aRowsPerItem + mtile * TC_M;
    const int bRow0 = item * p.bRowsPerItem + (int)rank * halfRows;
    const int nValid = p.nTotal > 0 ? min(p.N, p.nTotal - item * p.N) : p.N;
    const int nkb = p.Kd / BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.stages; s++) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 2);
        }
        mbar_init(accum, 1);
        *abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
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
    // the peer's barriers are initialised before any copy or commit reaches them
    cluster_sync_all();

    int issuedTma = 0, issuedMma = 0;
    if (warp == 0 && lane == 0) {
        for (int kb = 0; kb < nkb; kb++) {
            const int s = kb % p.stages;
            const int round = kb / p.stages;
            if (round > 0 && !mbar_wait(empty + s, (round - 1) & 1, kWaitBudget)) {
                atomicOr(p.flag, 4);
                *(volatile int*)abortFlag = 1;
                break;
            }
            if (*(volatile int*)abortFlag) break;
            uint8_t* st = smem + s * stageBytes;
            mbar_expect_tx(full + s, stageBytes);
            tma_load_2d(st, &tmAh, full + s, kb * BK, aRow0);
            tma_load_2d(st + aBytes, &tmAl, full + s, kb * BK, aRow0);
            uint8_t* bh = st + 2 * aBytes + (size_t)rank * halfRows * BK * 2;
            tma_load_2d_mc(bh, &tmBh, full + s, kb * BK, bRow0, both);
            tma_load_2d_mc(bh + bBytes, &tmBl, full + s, kb * BK, bRow0, both);
            issuedTma = kb + 1;
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = umma_idesc(TC_M, p.ntile);
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
            const uint32_t bh = smem_u32(st + 2 * aBytes), bl = smem_u32(st + 2 * aBytes + bBytes);
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++) {
                const uint32_t off = kk * 32;
                umma_bf16(tmem, desc<BK>(ah + off), desc<BK>(bh + off), idesc,
                          (kb | kk) != 0);
                umma_bf16(tmem, desc<BK>(ah + off), desc<BK>(bl + off), idesc, 1);
                umma_bf16(tmem, desc<BK>(al + off), desc<BK>(bh + off), idesc, 1);
            }
            umma_commit_mc(empty + s, both);     // frees the stage in both CTAs' count
            issuedMma = kb + 1;
        }
        umma_commit(accum);
    }
    __syncthreads();
    bool ok = *(volatile int*)abortFlag == 0 && mbar_wait(accum, 0, kWaitBudget);
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) {
        atomicOr(p.flag, 4);
        *(volatile int*)abortFlag = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool aborted = !ok;
    if (!aborted) {
        // every copy into this CTA's stages has landed (its MMAs read them all)
        const int pitch = p.ntile + 1;
        float* stage = reinterpret_cast<float*>(smem) + (size_t)warp * 32 * pitch;
        const int rowBase = mtile * TC_M + warp * 32;
        const bool rowOk = rowBase + lane < p.M;
        const float add = (rowOk && p.nrm) ? p.nrm[item * p.sN + rowBase + lane] : 0.f;
        for (int c0 = 0; c0 < p.ntile; c0 += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int i = 0; i < 16; i++) stage[lane * pitch + c0 + i] = fmaf(p.alpha, v[i], add);
        }
        __syncwarp();
        float* cbase = p.C + item * p.sC;
        for (int rr = 0; rr < 32; rr++) {
            const int r = rowBase + rr;
            if (r >= p.M) break;
            for (int j = lane; j < nValid; j += 32) {
                size_t off;
                if (p.cGroup > 0) {
                    const int jj = item * p.colPerItem + j;
                    const int l = jj / p.cGroup;
                    off = (size_t)l * p.cGroupStride + (size_t)r * p.ldc + (jj - l * p.cGroup);
                } else {
                    off = (size_t)r * p.ldc + j;
                }
                cbase[off] = stage[rr * pitch + j];
            }
        }
    }
    if (aborted && warp == 0 && lane == 0) {
        for (int kb = 0; kb < issuedTma; kb++) {
            const int s = kb % p.stages;
            mbar_wait(full + s, (kb / p.stages) & 1, kWaitBudget / 4);
        }
    }
    if (aborted && warp == 1 && lane == 0 && issuedMma > 0)
        mbar_wait(accum, 0, kWaitBudget / 4);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(p.tmemCols)
                     : "memory");
    }
    // neither CTA leaves while the other may still signal it
    cluster_sync_all();
}

}  // namespace

bool bf16x3_available() { return tc::encode_fn() != nullptr; }

size_t bf16x3_scratch_bytes(int, int, int, int) { return 256; }

// A and B point at the hi planes; the lo plane of each follows its hi plane
// (rows * Kd bf16 elements later).  lda / ldb must equal Kd.
// General form.  A: hi plane at A, lo plane rowsA x Kd elements later; B the
// same with rowsB.  Item i uses A rows i * aRowsPerItem + (0 .. M) and B rows
// i * bRowsPerItem + (0 .. N); it writes C + i * sC (+ row * ldc + col) for
// row < M and col < N (col < nTotal - i * N when nTotal > 0).
cudaError_t launch_gemm_bf16x3(const void* A, long long rowsA, const void* B, long long rowsB,
                               int M, int N, int Kd, int items, int aRowsPerItem,
                               int bRowsPerItem, int nTotal, float* C, long long sC, int ldc,
                               const float* nrm, long long sN, float alpha, int* flag,
                               cudaStream_t st, int cGroup, long long cGroupStride, bool pair,
                               int bk)
{
    if (bk != 64 && bk != 32) return cudaErrorInvalidValue;
    if (N <= 0 || N > 256 || M <= 0 || items <= 0 || Kd <= 0 || Kd % bk)
        return cudaErrorInvalidValue;
    const __nv_bfloat16* Ah = reinterpret_cast<const __nv_bfloat16*>(A);
    const __nv_bfloat16* Al = Ah + rowsA * Kd;
    const __nv_bfloat16* Bh = reinterpret_cast<const __nv_bfloat16*>(B);
    const __nv_bfloat16* Bl = Bh + rowsB * Kd;
    TcParams p;
    p.M = M;
    p.N = N;
    p.Kd = Kd;
    p.aRowsPerItem = aRowsPerItem;
    p.bRowsPerItem = bRowsPerItem;
    p.nTotal = nTotal;
    p.colPerItem = N;
    p.cGroup = cGroup;
    p.cGroupStride = cGroupStride;
    p.ntile = (N + 15) / 16 * 16;
    p.tmemCols = 32;
    while (p.tmemCols < p.ntile) p.tmemCols <<= 1;
    const int stageBytes = 2 * TC_M * bk * 2 + 2 * p.ntile * bk * 2;
    p.stages = (200 * 1024) / stageBytes;
    const int maxStages = bk == 64 ? 4 : 6;
    if (p.stages > maxStages) p.stages = maxStages;
    if (p.stages < 2) return cudaErrorInvalidValue;
    // the epilogue stages 128 rows of ntile + 1 floats in the pipeline buffers
    if ((size_t)TC_M * (p.ntile + 1) * 4 > (size_t)p.stages * stageBytes) return cudaErrorInvalidValue;
    p.C = C;
    p.sC = sC;
    p.ldc = ldc;
    p.nrm = nrm;
    p.sN = sN;
    p.alpha = alpha;
    p.flag = flag;
    const bool sw64 = bk == 32;
    CUtensorMap mAh, mAl, mBh, mBl;
    if (!tc::make_map(&mAh, Ah, rowsA, Kd, TC_M, bk, sw64) ||
        !tc::make_map(&mAl, Al, rowsA, Kd, TC_M, bk, sw64) ||
        !tc::make_map(&mBh, Bh, rowsB, Kd, p.ntile, bk, sw64) ||
        !tc::make_map(&mBl, Bl, rowsB, Kd, p.ntile, bk, sw64))
        return cudaErrorInvalidValue;
    const size_t smem = 1024 + (size_t)p.stages * stageBytes + 256;
    const int mTiles = (M + TC_M - 1) / TC_M;
    if (pair && mTiles >= 2) {
        // CTA pairs on neighbouring row tiles (an odd count gets a tile of
        // rows past M, zero-filled by TMA and not stored); each loads half of
        // the B rows, multicast to both
        CUtensorMap hBh, hBl;
        if (!tc::make_map(&hBh, Bh, rowsB, Kd, p.ntile / 2, bk, sw64) ||
            !tc::make_map(&hBl, Bl, rowsB, Kd, p.ntile / 2, bk, sw64))
            return cudaErrorInvalidValue;
        void (*kern)(const CUtensorMap, const CUtensorMap, const CUtensorMap, const CUtensorMap,
                     const TcParams) = bk == 64 ? k_gemm_bf16x3_pair<64> : k_gemm_bf16x3_pair<32>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)((mTiles + 1) / 2 * 2), (unsigned)items);
        cfg.blockDim = dim3(TC_THREADS);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, kern, mAh, mAl, hBh, hBl, p);
    }
    void (*kern)(const CUtensorMap, const CUtensorMap, const CUtensorMap, const CUtensorMap,
                 const TcParams) = bk == 64 ? k_gemm_bf16x3<64> : k_gemm_bf16x3<32>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(mTiles, items);
    kern<<<grid, TC_THREADS, smem, st>>>(mAh, mAl, mBh, mBl, p);
    return cudaGetLastError();
}

// Batched form: item b multiplies A rows [b M, (b + 1) M) with B rows
// [b N, (b + 1) N).  lda / ldb must equal Kd and the batch strides M Kd / N Kd.
cudaError_t launch_gemm_nt_bf16x3(const float* A, long long sA, int lda, const float* B,
                                  long long sB, int ldb, int M, int N, int Kd, int batch,
                                  float* C, long long sC, int ldc, const float* nrm,
                                  long long sN, float alpha, void*, size_t, int* flag,
                                  cudaStream_t st, int bk)
{
    if (lda != Kd || ldb != Kd || sA != (long long)M * Kd || sB != (long long)N * Kd)
        return cudaErrorInvalidValue;
    return launch_gemm_bf16x3(A, (long long)batch * M, B, (long long)batch * N, M, N, Kd, batch, M,
                              N, 0, C, sC, ldc, nrm, sN, alpha, flag, st, 0, 0, false,
                              Kd % bk == 0 ? bk : 64);
}

}  // namespace tg3
