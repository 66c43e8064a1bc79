// tg3_conv_tc.cu -- the pose network's inference forward with bf16
// activations: every 3x3 convolution with 32 or more input channels, and the
// 8192 -> 256 dense layer (a 1x1 convolution of a 1x1 image), as an implicit
// GEMM on the 5th-generation tensor cores; the first convolution (one input
// channel) and the 256 -> 68 output layer on CUDA cores.
//
// A split-K launch (the dense layer: few output rows, a long K) gives each
// CTA of grid row y a slice of the K blocks and writes FP32 partial sums,
// added in slice order by k_splitk_reduce with the bias and ReLU.
//
// Implicit GEMM: M = output pixels (images x rows x columns, NHWC order),
// N = output channels, K = taps x input channels (tap-major).  A CTA takes
// 128 output pixels and all N channels; per K block of 32 bf16 (one tap,
// 32 channels of it) its threads gather the A tile from the NHWC input (the
// zero padding of the convolution is a zero row segment) and copy the B tile
// of the repacked weights, both into shared memory in the 64-byte-swizzle
// K-major layout; one thread issues two 128 x N x 16 MMAs into a TMEM
// accumulator.  Two stages: the threads fill one while the tensor cores read
// the other.  The epilogue adds the bias, applies ReLU and stores bf16 NHWC.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "tg3_internal.cuh"
#include "tg3_tcgen05.cuh"

namespace tg3 {
namespace {

using namespace tc;

constexpr int CT_M = 128;        // output pixels per CTA
constexpr int CT_BK = 32;        // K (bf16) per stage: 64-byte rows
constexpr int CT_THREADS = 256;
constexpr int CT_ABYTES = CT_M * CT_BK * 2;

__device__ __forceinline__ uint32_t swz64(int r, int b)
{
    return (uint32_t)((r >> 3) * 512 + (r & 7) * 64 +
                      ((((b >> 4) ^ ((r >> 1) & 3)) << 4) | (b & 15)));
}

__global__ void __launch_bounds__(CT_THREADS, 4)
k_conv_tc(ConvTcArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int bBytes = a.coutPad * CT_BK * 2;
    const int stageBytes = CT_ABYTES + bBytes;
    uint64_t* empty = reinterpret_cast<uint64_t*>(smem + 2 * stageBytes);   // [2]
    uint64_t* accum = empty + 2;
    uint64_t* drain = empty + 3;
    uint32_t* tmemSlot = reinterpret_cast<uint32_t*>(empty + 4);
    int* abortp = reinterpret_cast<int*>(tmemSlot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0) {
        mbar_init(empty + 0, 1);
        mbar_init(empty + 1, 1);
        mbar_init(accum, 1);
        mbar_init(drain, 1);
        *abortp = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmemSlot)),
                     "r"(a.tmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmemSlot;

    const long long M = (long long)a.n * a.Ho * a.Wo;
    const long long m0 = (long long)blockIdx.x * CT_M;
    // this thread's A row (output pixel) and its 32-byte half of the row
    const int r = tid >> 1, hh = tid & 1;
    const long long m = m0 + r;
    const bool rowOk = m < M;
    int img = 0, oy = 0, ox = 0;
    if (rowOk) {
        const int hw = a.Ho * a.Wo;
        img = (int)(m / hw);
        const int rem = (int)(m % hw);
        oy = rem / a.Wo;
        ox = rem % a.Wo;
    }
    const int taps = a.ks * a.ks;
    // this CTA's K blocks: all, or its slice of a split-K launch
    const int nkbAll = a.Kpad / CT_BK;
    const int per = (nkbAll + a.kSplit - 1) / a.kSplit;
    const int kbBeg = blockIdx.y * per;
    const int nkb = min(nkbAll, kbBeg + per) - kbBeg;
    const uint32_t idesc = umma_idesc(CT_M, a.coutPad);
    bool issued = false;
    // the next block's A and B pieces, loaded a block ahead into registers
    uint4 v0, v1, wb[4];
    auto load_block = [&](int kb) {
        const int k0 = (kbBeg + kb) * CT_BK;
        const int tap = k0 / a.Cin;
        const int ci = k0 - tap * a.Cin + 16 * hh;
        v0 = make_uint4(0u, 0u, 0u, 0u);
        v1 = v0;
        if (rowOk && tap < taps) {
            const int ky = tap / a.ks, kx = tap - (tap / a.ks) * a.ks;
            const int iy = oy * a.stride + ky - a.pad, ix = ox * a.stride + kx - a.pad;
            if (iy >= 0 && iy < a.H && ix >= 0 && ix < a.W) {
                const uint4* src = reinterpret_cast<const uint4*>(
                    a.in + (((size_t)img * a.H + iy) * a.W + ix) * a.Cin + ci);
                v0 = __ldg(src);
                v1 = __ldg(src + 1);
            }
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int u = tid + i * CT_THREADS;
            if (u < a.coutPad * 4)
                wb[i] = __ldg(reinterpret_cast<const uint4*>(a.w + (size_t)(u >> 2) * a.Kpad + k0) +
                              (u & 3));
        }
    };
    if (nkb > 0) load_block(0);
    for (int kb = 0; kb < nkb; kb++) {
        const int s = kb & 1;
        uint8_t* st = smem + s * stageBytes;
        // the MMAs of block kb - 2 read this stage
        if (kb >= 2 && tid == 0 && !mbar_wait(empty + s, ((kb - 2) >> 1) & 1, kWaitBudget))
            *abortp = 1;
        __syncthreads();
        if (*abortp) break;
        // A: 16 channels of one tap for this row; B: the block's 32 K columns
        // of every output channel
        *reinterpret_cast<uint4*>(st + swz64(r, 32 * hh)) = v0;
        *reinterpret_cast<uint4*>(st + swz64(r, 32 * hh + 16)) = v1;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int u = tid + i * CT_THREADS;
            if (u < a.coutPad * 4)
                *reinterpret_cast<uint4*>(st + CT_ABYTES + swz64(u >> 2, 16 * (u & 3))) = wb[i];
        }
        if (kb + 1 < nkb) load_block(kb + 1);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(st), sb = smem_u32(st + CT_ABYTES);
#pragma unroll
            for (int kk = 0; kk < CT_BK / 16; kk++)
                umma_bf16(tmem, umma_desc_sw64(sa + 32 * kk), umma_desc_sw64(sb + 32 * kk), idesc,
                          (kb | kk) != 0);
            umma_commit(empty + s);
            if (kb == nkb - 1) umma_commit(accum);
        }
        issued = true;
    }
    if (tid == 0 && !*abortp && nkb > 0 && !mbar_wait(accum, 0, kWaitBudget)) *abortp = 1;
    __syncthreads();
    const bool ok = !*abortp;
    if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int quarter = warp & 3, colHalf = warp >> 2;
        const int row = 32 * quarter + lane;
        const long long mo = m0 + row;
        for (int c0 = 16 * colHalf; c0 < a.coutPad; c0 += 32) {
            float v[16];
            if (nkb > 0) {
                tmem_ld16(tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int i = 0; i < 16; i++) v[i] = 0.f;
            }
            if (a.partial && mo < M && c0 < a.Cout) {
                // split-K: this slice's sums, reduced by k_splitk_reduce
                float4* dst = reinterpret_cast<float4*>(
                    a.partial + ((size_t)blockIdx.y * M + mo) * a.Cout + c0);
#pragma unroll
                for (int i = 0; i < 4; i++)
                    dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            } else if (mo < M && c0 < a.Cout) {
                uint32_t pk[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    float x0 = v[2 * i] + __ldg(a.bias + c0 + 2 * i);
                    float x1 = v[2 * i + 1] + __ldg(a.bias + c0 + 2 * i + 1);
                    if (a.relu) {
                        x0 = fmaxf(x0, 0.f);
                        x1 = fmaxf(x1, 0.f);
                    }
                    const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
                    pk[i] = *reinterpret_cast<const uint32_t*>(&h);
                }
                uint4* dst = reinterpret_cast<uint4*>(a.out + (size_t)mo * a.Cout + c0);
                dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
        }
    } else if (tid == 0) {
        atomicOr(a.flag, 4);
        if (issued) {
            // let this CTA's own MMAs finish before the tensor memory is freed
            umma_commit(drain);
            mbar_wait(drain, 0, kWaitBudget / 4);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(a.tmemCols)
                     : "memory");
    }
}

// First layer: one input channel (the FP32 image, read as bf16), 3x3, pad 1,
// stride 1, 32 outputs with ReLU; one thread per output pixel, NHWC bf16.
__global__ void __launch_bounds__(256)
k_conv1_nhwc(const float* __restrict__ img, const __nv_bfloat16* __restrict__ w,
             const float* __restrict__ bias, int n, int H, __nv_bfloat16* __restrict__ out)
{
    __shared__ float ws[32 * 9];
    __shared__ float bs[32];
    for (int i = threadIdx.x; i < 32 * 9; i += blockDim.x) ws[i] = __bfloat162float(w[i]);
    if (threadIdx.x < 32) bs[threadIdx.x] = bias[threadIdx.x];
    __syncthreads();
    const long long npx = (long long)n * H * H;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npx;
         p += (long long)gridDim.x * blockDim.x) {
        const int im = (int)(p / (H * H));
        const int rem = (int)(p % (H * H));
        const int y = rem / H, x = rem % H;
        float t[9];
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const int iy = y + k / 3 - 1, ix = x + k % 3 - 1;
            const float v = (iy >= 0 && iy < H && ix >= 0 && ix < H)
                                ? img[((size_t)im * H + iy) * H + ix] : 0.f;
            t[k] = __bfloat162float(__float2bfloat16_rn(v));
        }
        uint4* dst = reinterpret_cast<uint4*>(out + (size_t)p * 32);
#pragma unroll 1
        for (int q = 0; q < 4; q++) {
            uint32_t pk[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                float a0 = bs[8 * q + 2 * i], a1 = bs[8 * q + 2 * i + 1];
#pragma unroll
                for (int k = 0; k < 9; k++) {
                    a0 = fmaf(ws[(8 * q + 2 * i) * 9 + k], t[k], a0);
                    a1 = fmaf(ws[(8 * q + 2 * i + 1) * 9 + k], t[k], a1);
                }
                const __nv_bfloat162 h = __floats2bfloat162_rn(fmaxf(a0, 0.f), fmaxf(a1, 0.f));
                pk[i] = *reinterpret_cast<const uint32_t*>(&h);
            }
            dst[q] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
    }
}

// Output layer: out[i][o] = bias[o] + sum_k W[o][k] act[i][k] (FP32 out).
// A CTA takes 8 images (their inputs in shared memory); a warp per output
// row of W, lanes along k (coalesced), one shuffle reduction per image.
constexpr int kFcImages = 8;

__global__ void __launch_bounds__(256)
k_fc_out(const __nv_bfloat16* __restrict__ act, const __nv_bfloat16* __restrict__ w,
         const float* __restrict__ bias, int n, int K, int N, float* __restrict__ out)
{
    extern __shared__ float xs[];                      // [kFcImages][K]
    const int i0 = blockIdx.x * kFcImages;
    const int ni = min(kFcImages, n - i0);
    for (int t = threadIdx.x; t < ni * K; t += blockDim.x)
        xs[t] = __bfloat162float(act[(size_t)i0 * K + t]);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int o = warp; o < N; o += blockDim.x >> 5) {
        float acc[kFcImages];
#pragma unroll
        for (int i = 0; i < kFcImages; i++) acc[i] = 0.f;
        for (int k = lane; k < K; k += 32) {
            const float wk = __bfloat162float(w[(size_t)o * K + k]);
#pragma unroll
            for (int i = 0; i < kFcImages; i++)
                if (i < ni) acc[i] = fmaf(wk, xs[i * K + k], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < kFcImages; i++) {
            float v = acc[i];
            for (int sft = 16; sft; sft >>= 1) v += __shfl_xor_sync(0xffffffffu, v, sft);
            if (lane == 0 && i < ni) out[(size_t)(i0 + i) * N + o] = v + bias[o];
        }
    }
}

// out[m][c] = bf16(act(sum over the slices of partial[s][m][c] + bias[c])),
// the slices in order.
__global__ void k_splitk_reduce(const float* __restrict__ partial, int kSplit, long long M,
                                int Cout, const float* __restrict__ bias, int relu,
                                __nv_bfloat16* __restrict__ out)
{
    const size_t n = (size_t)M * Cout;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int s = 0; s < kSplit; s++) acc += partial[(size_t)s * n + i];
        acc += bias[i % Cout];
        if (relu) acc = fmaxf(acc, 0.f);
        out[i] = __float2bfloat16_rn(acc);
    }
}

}  // namespace

size_t conv_tc_smem(int coutPad)
{
    return 1024 + 2 * (size_t)(CT_ABYTES + coutPad * CT_BK * 2) + 64;
}

cudaError_t launch_conv_tc(const ConvTcArgs& a, cudaStream_t st)
{
    if (a.Cin % CT_BK || a.Kpad % CT_BK || a.Kpad < a.ks * a.ks * a.Cin || a.coutPad % 16 ||
        a.Cout % 16 || a.Cout > a.coutPad ||
        a.coutPad < 16 || a.coutPad > 256 || a.tmemCols < a.coutPad)
        return cudaErrorInvalidValue;
    const size_t smem = conv_tc_smem(a.coutPad);
    cudaError_t e = cudaFuncSetAttribute(k_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    if (a.kSplit < 1 || a.kSplit > 65535 || (a.kSplit > 1 && !a.partial))
        return cudaErrorInvalidValue;
    const long long M = (long long)a.n * a.Ho * a.Wo;
    const long long grid = (M + CT_M - 1) / CT_M;
    if (grid <= 0 || grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    k_conv_tc<<<dim3((unsigned)grid, (unsigned)a.kSplit), CT_THREADS, smem, st>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess || !a.partial) return e;
    const size_t n = (size_t)M * a.Cout;
    k_splitk_reduce<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, st>>>(
        a.partial, a.kSplit, M, a.Cout, a.bias, a.relu, a.out);
    return cudaGetLastError();
}

cudaError_t launch_conv1_nhwc(const float* img, const __nv_bfloat16* w, const float* bias, int n,
                              int H, __nv_bfloat16* out, cudaStream_t st)
{
    const long long npx = (long long)n * H * H;
    const long long g = std::min<long long>((npx + 255) / 256, 152LL * 16);
    k_conv1_nhwc<<<(unsigned)g, 256, 0, st>>>(img, w, bias, n, H, out);
    return cudaGetLastError();
}

cudaError_t launch_fc_out(const __nv_bfloat16* act, const __nv_bfloat16* w, const float* bias,
                          int n, int K, int N, float* out, cudaStream_t st)
{
    const size_t smem = sizeof(float) * kFcImages * (size_t)K;
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    k_fc_out<<<(n + kFcImages - 1) / kFcImages, 256, smem, st>>>(act, w, bias, n, K, N, out);
    return cudaGetLastError();
}

}  // namespace tg3
