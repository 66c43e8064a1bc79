// tg3_noalloc.cu -- the local scoring of one particle without allocating.
//
// Who needs this: a caller that has handed all of a GPU's memory to its own
// pool allocator (an application that manages device memory itself), or that
// drives the E-step from many host threads at once (the reference's
// Optimiser scores particles from OpenMP threads), cannot let the library
// call cudaMalloc / cudaFree: those calls take memory the caller has already
// budgeted and they synchronise the device, stalling every other thread's
// work.  This entry point computes what tg3_local_phase_d computes for one
// particle (FP32 path) using a fixed scratch area that is part of the
// library image itself, so it allocates nothing.
//
// The scratch is one file-scope device array of kScratchBytes bytes.  Every
// GPU that loads the library holds it until the process exits.  All calls on
// a device share it, and it keeps the last call's contents:
//   - calls that can overlap on the GPU (different streams, or different host
//     threads without ordering) race on it and must not be issued;
//   - every call writes every scratch element it later reads (projection
//     rows and their zero padding, the shifted data, the likelihoods, the
//     norms and the error word), so no stale content from an earlier call is
//     used.
#include <cuda.h>   // CUcontext / CUresult types only; the driver is reached through cudart
#include <cuda_runtime.h>
#include <math_constants.h>

#include <mutex>

#include "tg3_internal.cuh"

namespace tg3 {

namespace {

constexpr size_t kScratchBytes = (size_t)64 << 20;   // 64 MiB

// scratch layout: [0, 256) error word, then the work arrays
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Projection of one particle's rotations from the plain complex half-FT
// volume (caller's layout, eight 8-byte corner loads per sample), with the
// row norm sum_p sigRcp ctf^2 |P|^2.  Trilinear weights and Friedel
// mirroring as in Volume::getByInterpolationFT (src/Image/Volume.cpp:308-332).
// A sample whose corners would fall outside the stored volume sets bit 16 of
// *flag and contributes zero.
__global__ void __launch_bounds__(256)
k_project_plain(const float2* __restrict__ vol, int vdim, int pf, const double* __restrict__ quat,
                const int* __restrict__ iCol, const int* __restrict__ iRow, int K,
                float* __restrict__ out, int ldo, const float* __restrict__ sigRcp,
                const float* __restrict__ ctf, float* __restrict__ nrm, int* __restrict__ flag)
{
    __shared__ float m[9];
    __shared__ float red[32];
    const int row = blockIdx.x;
    if (threadIdx.x == 0) {
        const double* q = quat + 4 * (size_t)row;
        const double A[3][3] = {{0, -q[3], q[2]}, {q[3], 0, -q[1]}, {-q[2], q[1], 0}};
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double aa = (2 * A[i][0]) * A[0][j] + (2 * A[i][1]) * A[1][j]
                          + (2 * A[i][2]) * A[2][j];
                m[3 * i + j] = (float)(((i == j ? 1.0 : 0.0) + (2 * q[0]) * A[i][j]) + aa);
            }
    }
    __syncthreads();
    const int nx = vdim / 2 + 1, half = vdim / 2;
    float2* orow = reinterpret_cast<float2*>(out + (size_t)row * ldo);
    float acc = 0.f;
    for (int p = threadIdx.x; p < ldo / 2; p += blockDim.x) {
        if (p >= K) {
            orow[p] = make_float2(0.f, 0.f);
            continue;
        }
        const float a = (float)iCol[p] * pf, b = (float)iRow[p] * pf;
        float x = m[0] * a + m[1] * b, y = m[3] * a + m[4] * b, z = m[6] * a + m[7] * b;
        const bool conj = x < 0.f;
        if (conj) { x = -x; y = -y; z = -z; }
        const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
        const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
        if (x0 + 1 > half || y0 < -half || y0 + 1 > half || z0 < -half || z0 + 1 > half) {
            atomicOr(flag, 1 << 16);
            orow[p] = make_float2(0.f, 0.f);
            continue;
        }
        const float fx = x - xf, fy = y - yf, fz = z - zf;
        const float wx[2] = {1.f - fx, fx}, wy[2] = {1.f - fy, fy}, wz[2] = {1.f - fz, fz};
        float re = 0.f, im = 0.f;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int zz = z0 + k < 0 ? z0 + k + vdim : z0 + k;
#pragma unroll
            for (int j = 0; j < 2; j++) {
                const int yy = y0 + j < 0 ? y0 + j + vdim : y0 + j;
                const float2* e = vol + ((size_t)zz * vdim + yy) * nx + x0;
                const float2 v0 = __ldg(e), v1 = __ldg(e + 1);
                const float w0 = wx[0] * wy[j] * wz[k], w1 = wx[1] * wy[j] * wz[k];
                re += v0.x * w0 + v1.x * w1;
                im += v0.y * w0 + v1.y * w1;
            }
        }
        if (conj) im = -im;
        orow[p] = make_float2(re, im);
        acc += sigRcp[p] * ctf[p] * ctf[p] * (re * re + im * im);
    }
    // block sum of the norm
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        nrm[row] = s;
    }
}

// Device address of the scratch array, looked up once per device and
// context.  The context's 64-bit id (cuCtxGetId, unique for the process's
// life) is kept with the address: after cudaDeviceReset the runtime makes a
// new primary context, reloads the library's module, and the array may sit
// at another address, so a changed id repeats the lookup.
using PfnCtxGetCurrent = CUresult (*)(CUcontext*);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long*);

struct ScratchSlot {
    unsigned long long ctx_id = 0;
    void* addr = nullptr;
};

std::mutex g_mu;
ScratchSlot g_slot[64];
std::once_flag g_driver_once;
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

int current_context_id(int dev, unsigned long long* id)
{
    std::call_once(g_driver_once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
            g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f);
    });
    if (!g_ctx_get_current || !g_ctx_get_id)
        return fail(TG3_ERR_CUDA, "driver entry points cuCtxGetCurrent / cuCtxGetId not found");
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS)
        return fail(TG3_ERR_CUDA, "cuCtxGetCurrent failed");
    if (!ctx) {
        // no context current on this thread yet: make the device's primary
        // context current (cudaSetDevice initialises it)
        TG3_CUDA(cudaSetDevice(dev));
        if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx)
            return fail(TG3_ERR_CUDA, "no CUDA context current after cudaSetDevice");
    }
    if (g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(TG3_ERR_CUDA, "cuCtxGetId failed");
    return TG3_OK;
}

int scratch_for_current_device(void** out)
{
    int dev = 0;
    TG3_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(TG3_ERR_ARG, "device ordinal out of range");
    unsigned long long id = 0;
    int st = current_context_id(dev, &id);
    if (st) return st;
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchSlot& s = g_slot[dev];
    if (!s.addr || s.ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(scratch)");
        s.addr = p;
        s.ctx_id = id;
    }
    *out = s.addr;
    return TG3_OK;
}

}  // namespace

}  // namespace tg3

using namespace tg3;

extern "C" size_t tg3_noalloc_scratch_bytes(void) { return kScratchBytes; }

extern "C" int tg3_local_phase_noalloc(const float* volume, int vdim, int pf, const int* iCol,
                                       const int* iRow, int K, int idim, const float* dat,
                                       const float* ctf, const float* sigRcp, const double* quat,
                                       int nR, const double* trans, int nT, const double* pwR,
                                       const double* pwT, const double* pwC, double* wC,
                                       double* wR, double* wT, double* baseL, float* dvp,
                                       void* stream)
{
    if (!volume || !iCol || !iRow || !dat || !ctf || !sigRcp || !quat || !trans || !pwR || !pwT ||
        !wC || !wR || !wT || !baseL)
        return fail(TG3_ERR_ARG, "null device pointer");
    if (vdim < 4 || (vdim & 1) || pf < 1 || K <= 0 || idim <= 0 || nR <= 0 || nT <= 0 ||
        nT > 2048)
        return fail(TG3_ERR_ARG, "bad sizes");
    const size_t Kp = round_up(2 * (size_t)K, 64);
    // layout after the 256-byte error word: P [nR][Kp], A [nT][Kp], D [nR][nT],
    // nrm [nR] (floats), x0 (double)
    const size_t offP = 256;
    const size_t offA = offP + round_up(sizeof(float) * nR * Kp, 256);
    const size_t offD = offA + round_up(sizeof(float) * nT * Kp, 256);
    const size_t offN = offD + round_up(sizeof(float) * (size_t)nR * nT, 256);
    const size_t offX = offN + round_up(sizeof(float) * nR, 256);
    const size_t need = offX + 256;
    if (need > kScratchBytes)
        return fail(TG3_ERR_ARG, "hypothesis set too large for the fixed scratch: needs " +
                                     std::to_string(need) + " bytes of " +
                                     std::to_string(kScratchBytes) +
                                     " ((nR + nT) x padded row + nR x nT floats)");
    void* base = nullptr;
    int st = scratch_for_current_device(&base);
    if (st) return st;
    char* s = static_cast<char*>(base);
    int* flag = reinterpret_cast<int*>(s);
    float* P = reinterpret_cast<float*>(s + offP);
    float* A = reinterpret_cast<float*>(s + offA);
    float* D = reinterpret_cast<float*>(s + offD);
    float* nrm = reinterpret_cast<float*>(s + offN);
    double* x0 = reinterpret_cast<double*>(s + offX);
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    TG3_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), cs));
    k_project_plain<<<nR, 256, 0, cs>>>(reinterpret_cast<const float2*>(volume), vdim, pf, quat,
                                         iCol, iRow, K, P, (int)Kp, sigRcp, ctf, nrm, flag);
    TG3_LAUNCH_CHECK("projection (no-alloc)");
    TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(dat), ctf, sigRcp, trans, nullptr, 1,
                               nT, idim, iCol, iRow, K, A, (int)Kp, 0, cs));
    TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(dat), sigRcp, 1, K, x0, cs));
    TG3_CUDA(launch_gemm_nt_fp32(P, 0, (int)Kp, A, 0, (int)Kp, nR, nT, (int)Kp, 1, D, 0, nT, nrm, 0,
                                 -2.0f, cs));
    TG3_CUDA(launch_weights(D, 0, nT, nR, nT, 1, 1, nullptr, 0, x0, pwR, 0, pwT, 0, pwC, wC, wR, wT,
                            baseL, dvp, cs));
    // the error word comes back on the call's own stream: a copy on the
    // legacy stream would also wait for every other blocking stream
    int h = 0;
    TG3_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, cs));
    TG3_CUDA(cudaStreamSynchronize(cs));
    if (h & (1 << 16))
        return fail(TG3_ERR_ARG, "a rotated pixel falls outside the volume (pf x radius too large)");
    return TG3_OK;
}
