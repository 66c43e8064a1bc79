// tg3_local2d.cu -- the local particle-filter scoring of 2-D classification.
//
// In 2-D mode the reference's local expectation (ExpectLocalV2D binds a
// class image, ExpectLocalRTD copies the particle's hypotheses -- in-plane
// rotations as (cos, sin) pairs -- and ExpectLocalPreI2D projects them,
// gpu/src/cuthunder.cu:2660-2810, kernel_Project2DL gpu/src/Kernel.cu:
// 750-778; ExpectLocalM then scores and sums the marginals) scores one
// particle against nR in-plane rotations of one class image x nT
// translations.  Here, per particle:
//   1. k_project2d samples the class image bilinearly at the rotated pixels
//      (Image::getByInterpolationFT, LINEAR_INTERP; Friedel mates
//      conjugated);
//   2. each row's norm sum_p sigRcp ctf^2 |P|^2 (k_norm_rows, FP64 sums of
//      FP32 terms);
//   3. the shifted, weighted data bank, the cross-term GEMM with the norm in
//      its epilogue, and the marginal weights -- the 3-D local phase's own
//      kernels.
#include <cuda_runtime.h>

#include <vector>

#include "tg3_internal.cuh"

struct tg3_image {
    tg3_ctx* ctx = nullptr;
    float2* img = nullptr;      // [vdim][vdim/2 + 1] complex, on the device
    int vdim = 0, pf = 0;
};

namespace tg3 {
namespace {

// nrm[r] = sum_p w[p] |P[r][p]|^2 with w = sigRcp ctf^2; one CTA per row.
__global__ void k_norm_rows(const float* __restrict__ P, int K, int ld,
                            const float* __restrict__ sigRcp, const float* __restrict__ ctf,
                            float* __restrict__ nrm)
{
    __shared__ double red[32];
    const float2* row = reinterpret_cast<const float2*>(P + (size_t)blockIdx.x * ld);
    double acc = 0.0;
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const float2 v = row[p];
        const float c = ctf[p];
        acc += (double)(sigRcp[p] * c * c * (v.x * v.x + v.y * v.y));
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
        nrm[blockIdx.x] = (float)s;
    }
}

}  // namespace
}  // namespace tg3

using namespace tg3;

extern "C" int tg3_image_create(tg3_image** out, const float* img, int vdim, int pf)
{
    if (!out || !img || vdim < 4 || (vdim & 1) || pf < 1)
        return fail(TG3_ERR_ARG, "bad class image arguments");
    *out = nullptr;
    int dev = 0;
    TG3_CUDA(cudaGetDevice(&dev));
    tg3_image* h = new tg3_image();
    int st = tg3_ctx_create(&h->ctx, dev);
    const size_t n = (size_t)vdim * (vdim / 2 + 1);
    if (st == TG3_OK && cudaMalloc(&h->img, sizeof(float2) * n) != cudaSuccess)
        st = fail(TG3_ERR_ALLOC, "class image allocation");
    if (st == TG3_OK &&
        cudaMemcpy(h->img, img, sizeof(float2) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        st = fail(TG3_ERR_CUDA, "class image upload");
    if (st != TG3_OK) {
        cudaFree(h->img);
        tg3_ctx_destroy(h->ctx);
        delete h;
        return st;
    }
    h->vdim = vdim;
    h->pf = pf;
    *out = h;
    return TG3_OK;
}

extern "C" int tg3_image_destroy(tg3_image* h)
{
    if (!h) return TG3_OK;
    if (h->ctx) cudaSetDevice(h->ctx->device);
    cudaFree(h->img);
    tg3_ctx_destroy(h->ctx);
    delete h;
    return TG3_OK;
}

extern "C" int tg3_ExpectLocal2D(tg3_image* h, const float* dat, const float* ctf,
                                 const float* sigRcp, const int* iCol, const int* iRow, int npxl,
                                 int idim, const double* rot, int nR, const double* trans, int nT,
                                 const double* oldR, const double* oldT, double oldC, float* wC,
                                 float* wR, float* wT, float* dvp, float* baseL)
{
    if (!h || !h->ctx || !h->img) return fail(TG3_ERR_ARG, "null class image handle");
    if (!dat || !ctf || !sigRcp || !iCol || !iRow || !rot || !trans || !oldR || !oldT || !wC ||
        !wR || !wT || !baseL || npxl <= 0 || nR <= 0 || nT <= 0 || nT > 2048)
        return fail(TG3_ERR_ARG, "bad ExpectLocal2D arguments");
    tg3_ctx* c = h->ctx;
    int st = check_ctx(c);
    if (st) return st;
    if (c->px.K != npxl || c->px.idim != idim) {
        if ((st = tg3_ctx_set_pixels(c, iCol, iRow, npxl, idim))) return st;
    }
    if ((st = check_geometry(c, h->vdim, h->pf))) return st;
    const int K = npxl, Kp = c->px.Kp;
    cudaStream_t s = c->stream;
    Arena ar(c, WS_H2D);
    const size_t od = ar.add(8 * (size_t)K), oc = ar.add(4 * (size_t)K),
                 os = ar.add(4 * (size_t)K), oq = ar.add(16 * (size_t)nR),
                 ot = ar.add(16 * (size_t)nT), opr = ar.add(8 * (size_t)nR),
                 opt = ar.add(8 * (size_t)nT), opc = ar.add(8), owc = ar.add(8),
                 owr = ar.add(8 * (size_t)nR), owt = ar.add(8 * (size_t)nT), obl = ar.add(8),
                 odv = ar.add(4 * (size_t)nR * nT), onr = ar.add(4 * (size_t)nR),
                 ox0 = ar.add(8);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    float* P = (float*)ws_get(c, WS_P, 4 * (size_t)nR * Kp, &st);
    if (!P) return st;
    float* A = (float*)ws_get(c, WS_A, 4 * (size_t)nT * Kp, &st);
    if (!A) return st;
    float* D = (float*)ws_get(c, WS_D, 4 * (size_t)nR * nT, &st);
    if (!D) return st;
    TG3_CUDA(cudaMemcpyAsync(b + od, dat, 8 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oc, ctf, 4 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + os, sigRcp, 4 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oq, rot, 16 * (size_t)nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ot, trans, 16 * (size_t)nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, oldR, 8 * (size_t)nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, oldT, 8 * (size_t)nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opc, &oldC, 8, cudaMemcpyHostToDevice, s));
    const float* dctf = (const float*)(b + oc);
    const float* dsig = (const float*)(b + os);
    float* nrm = (float*)(b + onr);
    double* x0 = (double*)(b + ox0);
    TG3_CUDA(launch_project2d(h->img, h->vdim, h->pf, (const double*)(b + oq), nR, c->px.iCol,
                              c->px.iRow, K, P, Kp, 0, s));
    k_norm_rows<<<nR, 256, 0, s>>>(P, K, Kp, dsig, dctf, nrm);
    TG3_LAUNCH_CHECK("row norms");
    TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(b + od), dctf, dsig,
                               (const double*)(b + ot), nullptr, 1, nT, idim, c->px.iCol,
                               c->px.iRow, K, A, Kp, 0, s));
    TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(b + od), dsig, 1, K, x0, s));
    TG3_CUDA(launch_gemm_nt_fp32(P, 0, Kp, A, 0, Kp, nR, nT, Kp, 1, D, 0, nT, nrm, 0, -2.0f, s));
    TG3_CUDA(launch_weights(D, 0, nT, nR, nT, 1, 1, nullptr, 0, x0, (const double*)(b + opr), 0,
                            (const double*)(b + opt), 0, (const double*)(b + opc),
                            (double*)(b + owc), (double*)(b + owr), (double*)(b + owt),
                            (double*)(b + obl), dvp ? (float*)(b + odv) : nullptr, s));
    std::vector<double> hwr(nR), hwt(nT);
    double hwc = 0, hbl = 0;
    TG3_CUDA(cudaMemcpyAsync(hwr.data(), b + owr, 8 * (size_t)nR, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(hwt.data(), b + owt, 8 * (size_t)nT, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hwc, b + owc, 8, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hbl, b + obl, 8, cudaMemcpyDeviceToHost, s));
    if (dvp) TG3_CUDA(cudaMemcpyAsync(dvp, b + odv, 4 * (size_t)nR * nT, cudaMemcpyDeviceToHost, s));
    if ((st = tg3_ctx_sync(c))) return st;
    for (int r = 0; r < nR; r++) wR[r] = (float)hwr[r];
    for (int t = 0; t < nT; t++) wT[t] = (float)hwt[t];
    *wC = (float)hwc;
    *baseL = (float)hbl;
    return TG3_OK;
}
