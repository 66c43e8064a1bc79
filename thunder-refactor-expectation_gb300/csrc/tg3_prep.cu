// Image preprocessing ahead of the expectation: real-space particle images
// to the complex pixel data the scoring kernels read (Optimiser::initImg,
// src/Optimiser.cpp:4600-4760, and allocPreCal, src/Optimiser.cpp:7995-8030).
// With r = maskRadius / pixelSize and centred coordinates (i, j), i, j in
// [-N/2, N/2) about the file's pixel (N/2, N/2):
//   substractBgImg (:4917): the mean m and standard deviation s (n - 1) of
//     the pixels with i^2 + j^2 > r^2 (bgMeanStddev, src/Image/
//     ImageFunctions.cpp:607-620); y = (x - m) / s;
//   statImg (:4796): stdN = the mean over the images of the same region's
//     standard deviation of y about 0 (bgStddev, ImageFunctions.cpp:585-596);
//   maskImg (:4953, zeroMask): y (u < r), y (1 - w) for r <= u <= r + 6 with
//     w = 0.5 - 0.5 cos((u - r) / 6 pi), 0 beyond (softMask, src/Functions/
//     Mask.cpp:363-385; EDGE_WIDTH_RL = 6); u = sqrt(i^2 + j^2);
//   normaliseImg (:4987): y / stdN;
//   fwImg (:5003): unnormalised forward r2c transform of the image with its
//     centre at index 0 (ImageFile's MESH_IMAGE_INDEX layout);
//   allocPreCal: dat[l][p] = FT at (iCol[p], iRow[p] mod N).
// The unmasked form (the reference's _imgOri) skips the mask.  The noise-
// filled mask of the non-zeroMask option draws from the reference's GSL
// random stream and is not offered.
#include <cufft.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {
namespace {

__device__ double prep_block_sum(double v, double* scratch)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double r = lane < nw ? scratch[lane] : 0.0;
        for (int o = 16; o; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
        if (lane == 0) scratch[0] = r;
    }
    __syncthreads();
    return scratch[0];
}

// Per-image background statistics: stats[l] = (m, s, sN), sN the background
// standard deviation of (x - m) / s about 0.  One pass: a warp per row, lanes
// over columns; each lane sums its pixels of a row about a pivot (the
// corner pixel, always background) in FP32 and adds the row's partial sums
// to FP64 totals.  Background: i^2 + j^2 > r^2, i.e. > floor(r^2) in
// integers.  CTA per image.
__global__ void __launch_bounds__(256)
k_bg_stats(const float* __restrict__ img, int N, long long bgAbove, double* __restrict__ st)
{
    __shared__ double red[32];
    const size_t l = blockIdx.x;
    const float* im = img + l * N * N;
    const int half = N / 2;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const float pivot = im[0];
    double s1 = 0.0, s2 = 0.0, cnt = 0.0;
    for (int y = warp; y < N; y += nw) {
        const int j = y - half;
        const float* row = im + (size_t)y * N;
        float a1 = 0.f, a2 = 0.f;
        int c = 0;
        for (int x = lane; x < N; x += 32) {
            const int i = x - half;
            if ((long long)(i * i + j * j) > bgAbove) {
                const float d = row[x] - pivot;
                a1 += d;
                a2 = fmaf(d, d, a2);
                c++;
            }
        }
        s1 += a1;
        s2 += a2;
        cnt += c;
    }
    s1 = prep_block_sum(s1, red);
    s2 = prep_block_sum(s2, red);
    cnt = prep_block_sum(cnt, red);
    if (threadIdx.x == 0) {
        const double mu = s1 / cnt;                 // mean about the pivot
        const double ss = fmax(s2 - s1 * mu, 0.0);  // sum of (x - m)^2
        const double sd = sqrt(ss / (cnt - 1.0));
        st[3 * l] = pivot + mu;
        st[3 * l + 1] = sd;
        // sum of ((x - m) / sd)^2 over the background, over (n - 1)
        st[3 * l + 2] = sqrt(ss / (sd * sd) / (cnt - 1.0));
    }
}

__global__ void k_stats_f32(const double* __restrict__ st, int n, float* __restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * n; i += gridDim.x * blockDim.x)
        out[i] = (float)st[i];
}

// stdN: the given value, or the mean of the images' sN; out = (stdN, 1 / stdN).
__global__ void k_stdn(const double* __restrict__ st, int n, float given, double* __restrict__ out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int l = threadIdx.x; l < n; l += blockDim.x) s += st[3 * (size_t)l + 2];
    s = prep_block_sum(s, red);
    if (threadIdx.x == 0) {
        out[0] = given > 0.f ? (double)given : s / n;
        out[1] = 1.0 / out[0];
    }
}

constexpr int kPrepRows = 4;   // image rows per CTA of k_prep_image

// Normalise, mask and scale one image row, written with the image's centre
// at index 0.
__global__ void k_prep_image(const float* __restrict__ img, int N, float r, float ew, int mask,
                             const double* __restrict__ st, const double* __restrict__ stdN,
                             float* __restrict__ out)
{
    const size_t l = blockIdx.y;
    const float m = (float)st[3 * l], sd = (float)st[3 * l + 1];
    const float scale = (float)stdN[1];
    const int half = N / 2;
    // CTA (kPrepRows rows, image l); threads over the rows' columns
    const int y1 = min(N, (int)(blockIdx.x + 1) * kPrepRows);
    for (int y = blockIdx.x * kPrepRows; y < y1; y++)
    for (int x = threadIdx.x; x < N; x += blockDim.x) {
        const int q = y * N + x;
        const int i = x - half, j = y - half;
        float v = (img[l * N * N + q] - m) / sd;
        if (mask) {
            const float u = sqrtf((float)(i * i + j * j));
            if (u > r + ew)
                v = 0.f;
            else if (u >= r) {
                const float w = 0.5f - 0.5f * cospif((u - r) / ew);
                v = v * (1.f - w);
            }
        }
        const int ci = i < 0 ? i + N : i, cj = j < 0 ? j + N : j;
        out[l * N * N + (size_t)cj * N + ci] = v * scale;
    }
}

// dat[l][p] = FT[l][iRow mod N][iCol]
__global__ void k_gather_pixels(const float2* __restrict__ ft, int N, const int* __restrict__ iCol,
                                const int* __restrict__ iRow, int K, float2* __restrict__ dat)
{
    const size_t l = blockIdx.y;
    const int nx = N / 2 + 1;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K; p += gridDim.x * blockDim.x) {
        const int row = iRow[p] < 0 ? iRow[p] + N : iRow[p];
        dat[l * K + p] = ft[(l * N + row) * nx + iCol[p]];
    }
}

// ------------------------------------------------------------ sigma^2 --
// Noise spectrum of the images against their best poses (Optimiser::
// allReduceSigma, src/Optimiser.cpp:6355-6630, with OPTIMISER_SIGMA_RANK1ST
// and OPTIMISER_SIGMA_WHOLE_FREQUENCY).  Per image l, with its model
// M = ctf P(R) S(t) and the unmasked model N = ctf P(R) S(t - offset) over the
// pixels of shells u = rint(|k|) < rSig (powerSpectrum, src/Functions/
// Spectrum.cpp:161-190, shell means):
//   vSigM[u] = <|datM - M|^2>, vSigN[u] = <|datN - N|^2>,
//   svd[u] = sqrt(<|M|^2> / <|datM|^2>);
// its group accumulates vSigM / 2, vSigN / 2, svd and a count.  CTA per
// image; shell sums in shared memory (FP32), group sums in FP64.
__global__ void __launch_bounds__(256)
k_sigma_image(const float2* __restrict__ P, int ldp, const float2* __restrict__ datM,
              const float2* __restrict__ datN, const float* __restrict__ ctf,
              const double* __restrict__ trans, const double* __restrict__ offset,
              const int* __restrict__ group, int byGroup, const int* __restrict__ iCol,
              const int* __restrict__ iRow, int K, int N, int rSig, double* __restrict__ acc)
{
    extern __shared__ float sh[];
    float* pM = sh;               // [rSig] each
    float* pN = pM + rSig;
    float* pS = pN + rSig;
    float* pD = pS + rSig;
    int* cnt = reinterpret_cast<int*>(pD + rSig);
    const size_t l = blockIdx.x;
    for (int u = threadIdx.x; u < rSig; u += blockDim.x) {
        pM[u] = pN[u] = pS[u] = pD[u] = 0.f;
        cnt[u] = 0;
    }
    __syncthreads();
    const float invN = 1.0f / (float)N;
    const float tx = (float)trans[2 * l], ty = (float)trans[2 * l + 1];
    const float ox = offset ? (float)offset[2 * l] : 0.f, oy = offset ? (float)offset[2 * l + 1] : 0.f;
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const int i = iCol[p], j = iRow[p];
        const int u = (int)rintf(sqrtf((float)(i * i + j * j)));
        if (u >= rSig || i * i + j * j >= rSig * rSig) continue;
        const float2 pr = P[l * ldp + p];
        const float c = ctf[l * K + p];
        float sn, cs;
        // S(t) = exp(-2 pi i (i tx + j ty) / N)
        sincospif(-2.0f * ((float)i * tx + (float)j * ty) * invN, &sn, &cs);
        const float mr = c * (pr.x * cs - pr.y * sn), mi = c * (pr.x * sn + pr.y * cs);
        float so, co;
        sincospif(2.0f * ((float)i * ox + (float)j * oy) * invN, &so, &co);
        const float nr = mr * co - mi * so, ni = mr * so + mi * co;   // S(t - offset)
        const float2 a = datM[l * K + p], b = datN[l * K + p];
        atomicAdd(pM + u, (a.x - mr) * (a.x - mr) + (a.y - mi) * (a.y - mi));
        atomicAdd(pN + u, (b.x - nr) * (b.x - nr) + (b.y - ni) * (b.y - ni));
        atomicAdd(pS + u, mr * mr + mi * mi);
        atomicAdd(pD + u, a.x * a.x + a.y * a.y);
        atomicAdd(cnt + u, 1);
    }
    __syncthreads();
    const int g = byGroup ? group[l] - 1 : 0;
    double* ag = acc + (size_t)g * (3 * rSig + 1);
    for (int u = threadIdx.x; u < rSig; u += blockDim.x) {
        const double n = (double)cnt[u];
        atomicAdd(ag + u, 0.5 * pM[u] / n);
        atomicAdd(ag + rSig + u, 0.5 * pN[u] / n);
        atomicAdd(ag + 2 * rSig + u, sqrt((double)pS[u] / (double)pD[u]));
    }
    if (threadIdx.x == 0) atomicAdd(ag + 3 * rSig, 1.0);
}

// sig = ratio sigM + (1 - ratio) alpha sigN, ratio = min(1, svd); all groups
// copy group 0 when the images were pooled.  One thread per (group, shell).
__global__ void k_sigma_finish(const double* __restrict__ acc, int nGroup, int rSig, int byGroup,
                               double alpha, double* __restrict__ sig, double* __restrict__ sigRcp)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nGroup * rSig) return;
    const int g = idx / rSig, u = idx % rSig;
    const double* ag = acc + (size_t)(byGroup ? g : 0) * (3 * rSig + 1);
    const double w = ag[3 * rSig];
    const double sM = ag[u] / w, sN = ag[rSig + u] / w, svd = ag[2 * rSig + u] / w;
    const double ratio = fmin(1.0, svd);
    const double s = ratio * sM + (1.0 - ratio) * alpha * sN;
    sig[idx] = s;
    sigRcp[idx] = -0.5 / s;
}

// batched r2c plans, one per (context, size, batch), kept until the context goes
struct Plan {
    tg3_ctx* c;
    int N, batch;
    cufftHandle h;
};
std::vector<Plan> g_plans;
std::mutex g_planLock;

// Batched 2-D plans of a context, forward (real to complex) or inverse.
int get_plan(tg3_ctx* c, int N, int batch, cufftHandle* out, bool inverse = false)
{
    std::lock_guard<std::mutex> g(g_planLock);
    const int key = inverse ? -batch : batch;
    for (auto& p : g_plans)
        if (p.c == c && p.N == N && p.batch == key) {
            *out = p.h;
            return TG3_OK;
        }
    cufftHandle h;
    int n[2] = {N, N};
    const cufftResult r =
        inverse ? cufftPlanMany(&h, 2, n, nullptr, 1, N * (N / 2 + 1), nullptr, 1, N * N,
                                CUFFT_C2R, batch)
                : cufftPlanMany(&h, 2, n, nullptr, 1, N * N, nullptr, 1, N * (N / 2 + 1),
                                CUFFT_R2C, batch);
    if (r != CUFFT_SUCCESS) return fail(TG3_ERR_CUDA, "cuFFT plan creation failed");
    g_plans.push_back({c, N, key, h});
    *out = h;
    return TG3_OK;
}

// ReMask's real-space step: x / N^2 (the normalisation of the inverse
// transform, FFT::bw) times the soft mask of radius r and edge ew about the
// centre at index 0 (kernel_SoftMask / kernel_MulMask, gpu/src/Kernel.cu:
// 5249-5316): 1 inside r, 0.5 + 0.5 cos((u - r) / ew pi) on the edge, 0
// beyond r + ew, u from the wrapped indices.
__global__ void k_remask_real(float* __restrict__ real, int N, float r, float ew, size_t n)
{
    const float inv = 1.0f / ((float)N * (float)N);
    const size_t per = (size_t)N * N;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n * per;
         q += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(q % N), y = (int)((q / N) % N);
        const int i = x < N / 2 ? x : x - N, j = y < N / 2 ? y : y - N;
        const float u = sqrtf((float)(i * i + j * j));
        const float m = u > r + ew ? 0.f : (u >= r ? 0.5f + 0.5f * cospif((u - r) / ew) : 1.f);
        real[q] = real[q] * inv * m;
    }
}

// The img x img rfft grid in the particle transforms' order: pixel
// p = r (img/2 + 1) + i holds column i and row j = r (r < img/2), r - img.
__global__ void k_image_grid(int img, int* __restrict__ iCol, int* __restrict__ iRow)
{
    const int h = img / 2, n = img * (h + 1);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int r = p / (h + 1), i = p % (h + 1);
        iCol[p] = i;
        iRow[p] = r < h ? r : r - img;
    }
}

// One CTA per image: the centred image (index 0 moved to the middle, as an
// fftshift), minus its mean, over its unbiased standard deviation; the sums
// in FP64.
__global__ void k_centre_normalise(const float* __restrict__ real, int img,
                                   float* __restrict__ out)
{
    __shared__ double s1[32], s2[32];
    const int n = img * img, h = img / 2;
    const float* src = real + (size_t)blockIdx.x * n;
    float* dst = out + (size_t)blockIdx.x * n;
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = src[i];
        a += v;
        b += v * v;
    }
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s1[threadIdx.x >> 5] = a;
        s2[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            ta += s1[w];
            tb += s2[w];
        }
        const double mean = ta / n;
        const double var = fmax((tb - ta * mean) / (n - 1), 0.0);
        s1[0] = mean;
        s2[0] = var > 0.0 ? 1.0 / sqrt(var) : 0.0;
    }
    __syncthreads();
    const double mean = s1[0], rs = s2[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int y = i / img, x = i % img;
        const int ys = y + h < img ? y + h : y + h - img, xs = x + h < img ? x + h : x + h - img;
        dst[(size_t)y * img + x] = (float)(((double)src[(size_t)ys * img + xs] - mean) * rs);
    }
}

}  // namespace

extern "C" int tg3_ctx_render_references_d(tg3_ctx* c, int cls, const double* rotMat, int n,
                                           int img, float* out)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks)
        return fail(TG3_ERR_STATE, "volume not set");
    if (!rotMat || !out || n <= 0 || img < 8 || (img & 1))
        return fail(TG3_ERR_ARG, "bad reference rendering arguments");
    const Volume& v = c->vol[cls];
    const int h = img / 2, K = img * (h + 1);
    // the grid's farthest pixel, (h, h) pf voxels out, with its trilinear
    // corners, must lie inside the stored half grid
    if ((int)ceil(1.41422 * h * v.pf) + 2 > v.vdim / 2)
        return fail(TG3_ERR_ARG, "reference image grid reaches past the volume");
    const int IB = std::min(n, 4096);
    const size_t oCol = 0, oRow = (sizeof(int) * K + 255) / 256 * 256,
                 oP = oRow + (sizeof(int) * K + 255) / 256 * 256,
                 oR = oP + (sizeof(float2) * (size_t)K * IB + 255) / 256 * 256,
                 total = oR + sizeof(float) * (size_t)img * img * IB;
    char* b = (char*)ws_get(c, WS_RENDER, total, &st);
    if (!b) return st;
    float* pscr = (float*)ws_get(c, WS_PROJ, sizeof(float) * project_scratch_floats(IB, 2 * K), &st);
    if (!pscr) return st;
    int* gCol = (int*)(b + oCol);
    int* gRow = (int*)(b + oRow);
    float* P = (float*)(b + oP);
    float* R = (float*)(b + oR);
    cudaStream_t s = c->stream;
    k_image_grid<<<(K + 255) / 256, 256, 0, s>>>(img, gCol, gRow);
    TG3_LAUNCH_CHECK("image grid");
    cufftHandle plan;
    for (int r0 = 0; r0 < n; r0 += IB) {
        const int m = std::min(IB, n - r0);
        TG3_CUDA(launch_project(nullptr, nullptr, v.blocks, v.vdim, v.pf, nullptr,
                                rotMat + 9 * (size_t)r0, m, m, gCol, gRow, K, P, 2 * K, nullptr,
                                nullptr, nullptr, pscr, c->d_flag, 0, s));
        if ((st = get_plan(c, img, m, &plan, true))) return st;
        if (cufftSetStream(plan, s) != CUFFT_SUCCESS ||
            cufftExecC2R(plan, reinterpret_cast<cufftComplex*>(P), R) != CUFFT_SUCCESS)
            return fail(TG3_ERR_CUDA, "cuFFT inverse transform failed");
        k_centre_normalise<<<m, 256, 0, s>>>(R, img, out + (size_t)r0 * img * img);
        TG3_LAUNCH_CHECK("reference centring");
    }
    return TG3_OK;
}

void prep_release(tg3_ctx* c)
{
    std::lock_guard<std::mutex> g(g_planLock);
    for (size_t i = 0; i < g_plans.size();) {
        if (g_plans[i].c == c) {
            cufftDestroy(g_plans[i].h);
            g_plans.erase(g_plans.begin() + i);
        } else {
            i++;
        }
    }
}

}  // namespace tg3

using namespace tg3;

extern "C" int tg3_sigma_d(tg3_ctx* c, int cls, int nImg, const float* datM, const float* datN,
                           const float* ctf, const double* rotMat, const double* trans,
                           const double* offset, const int* group, int nGroup, int byGroup,
                           int rSig, float maskRadius, float pixelSize, double* sig,
                           double* sigRcp)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks)
        return fail(TG3_ERR_STATE, "volume of the class not set");
    if (!datM || !datN || !ctf || !rotMat || !trans || !sig || !sigRcp || (byGroup && !group))
        return fail(TG3_ERR_ARG, "null device pointer");
    if (nImg <= 0 || nGroup <= 0 || rSig <= 0 || rSig > 2048 || !(pixelSize > 0))
        return fail(TG3_ERR_ARG, "bad sigma arguments");
    const Volume& v = c->vol[cls];
    if ((st = check_geometry(c, v.vdim, v.pf))) return st;
    const int K = c->px.K, N = c->px.idim;
    if (rSig > N / 2) return fail(TG3_ERR_ARG, "rSig beyond the image's Nyquist shell");
    const int IB = std::min(nImg, 2048);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t accN = (size_t)nGroup * (3 * rSig + 1);
    const size_t oA = 0, oP = up(sizeof(double) * accN), total = oP + sizeof(float2) * (size_t)K * IB;
    char* b = (char*)ws_get(c, WS_PREP, total, &st);
    if (!b) return st;
    double* acc = (double*)(b + oA);
    float* P = (float*)(b + oP);
    float* pscr = (float*)ws_get(c, WS_PROJ, sizeof(float) * project_scratch_floats(IB, 2 * K), &st);
    if (!pscr) return st;
    cudaStream_t s = c->stream;
    TG3_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * accN, s));
    const size_t smem = (4 * sizeof(float) + sizeof(int)) * (size_t)rSig;
    for (int l0 = 0; l0 < nImg; l0 += IB) {
        const int n = std::min(IB, nImg - l0);
        TG3_CUDA(launch_project(nullptr, nullptr, v.blocks, v.vdim, v.pf, nullptr,
                                rotMat + 9 * (size_t)l0, n, n, c->px.iCol, c->px.iRow, K, P, 2 * K,
                                nullptr, nullptr, nullptr, pscr, c->d_flag, 0, s));
        const size_t o = (size_t)l0 * K;
        k_sigma_image<<<n, 256, smem, s>>>(
            reinterpret_cast<const float2*>(P), K, reinterpret_cast<const float2*>(datM) + o,
            reinterpret_cast<const float2*>(datN) + o, ctf + o, trans + 2 * (size_t)l0,
            offset ? offset + 2 * (size_t)l0 : nullptr, byGroup ? group + l0 : nullptr, byGroup,
            c->px.iCol, c->px.iRow, K, N, rSig, acc);
        TG3_LAUNCH_CHECK("sigma per image");
    }
    const double rm = (double)maskRadius / ((double)N * (double)pixelSize);
    const double alpha = sqrt(M_PI * rm * rm);
    k_sigma_finish<<<(nGroup * rSig + 255) / 256, 256, 0, s>>>(acc, nGroup, rSig, byGroup, alpha,
                                                                sig, sigRcp);
    TG3_LAUNCH_CHECK("sigma finish");
    return TG3_OK;
}

extern "C" int tg3_prepare_images_d(tg3_ctx* c, const float* img, int nImg, int N,
                                    float maskRadiusPx, int mask, float stdN, float* dat,
                                    float* stats)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!img || !dat || nImg <= 0 || N < 4 || (N & 1) || !(maskRadiusPx > 0))
        return fail(TG3_ERR_ARG, "bad preprocessing arguments");
    if (!c->px.iCol || c->px.idim != N)
        return fail(TG3_ERR_STATE, "the active pixel set was not made for this image size");
    if (maskRadiusPx >= N / 2 * 1.4142135f)
        return fail(TG3_ERR_ARG, "mask radius leaves no background pixels");
    const int K = c->px.K;
    const int IB = std::min(nImg, 2048);
    const size_t img2 = (size_t)N * N, ft2 = (size_t)N * (N / 2 + 1);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t oSt = 0, oN = up(sizeof(double) * 3 * (size_t)nImg), oR = oN + 256,   // oN: 2 doubles
                 oF = up(oR + sizeof(float) * img2 * IB), total = oF + sizeof(float2) * ft2 * IB;
    char* b = (char*)ws_get(c, WS_PREP, total, &st);
    if (!b) return st;
    double* stv = (double*)(b + oSt);
    double* sN = (double*)(b + oN);
    float* real = (float*)(b + oR);
    cufftComplex* ft = (cufftComplex*)(b + oF);
    cudaStream_t s = c->stream;
    const float r = maskRadiusPx;
    k_bg_stats<<<nImg, 256, 0, s>>>(img, N, (long long)std::floor((double)r * (double)r), stv);
    TG3_LAUNCH_CHECK("background statistics");
    k_stdn<<<1, 256, 0, s>>>(stv, nImg, stdN, sN);
    TG3_LAUNCH_CHECK("noise level");
    for (int l0 = 0; l0 < nImg; l0 += IB) {
        const int n = std::min(IB, nImg - l0);
        k_prep_image<<<dim3((N + kPrepRows - 1) / kPrepRows, n), std::min(N, 256), 0, s>>>(
            img + (size_t)l0 * img2, N, r, 6.0f, mask, stv + 3 * (size_t)l0, sN, real);
        TG3_LAUNCH_CHECK("normalise and mask");
        cufftHandle h;
        if ((st = get_plan(c, N, n, &h))) return st;
        if (cufftSetStream(h, s) != CUFFT_SUCCESS || cufftExecR2C(h, real, ft) != CUFFT_SUCCESS)
            return fail(TG3_ERR_CUDA, "cuFFT forward transform failed");
        k_gather_pixels<<<dim3((K + 255) / 256, n), 256, 0, s>>>(
            reinterpret_cast<const float2*>(ft), N, c->px.iCol, c->px.iRow, K,
            reinterpret_cast<float2*>(dat) + (size_t)l0 * K);
        TG3_LAUNCH_CHECK("pixel gather");
    }
    if (stats) {
        k_stats_f32<<<(3 * nImg + 255) / 256, 256, 0, s>>>(stv, nImg, stats);
        TG3_LAUNCH_CHECK("statistics");
    }
    return TG3_OK;
}

extern "C" int tg3_remask_d(tg3_ctx* c, const float* imgFT, int nImg, int N, float maskRadiusPx,
                            float edgeWidth, float* out)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!imgFT || !out || nImg <= 0 || N < 4 || (N & 1) || !(maskRadiusPx > 0) ||
        !(edgeWidth > 0))
        return fail(TG3_ERR_ARG, "bad re-mask arguments");
    const int IB = std::min(nImg, 2048);
    const size_t img2 = (size_t)N * N, ft2 = (size_t)N * (N / 2 + 1);
    // the inverse transform overwrites its input: it reads a copy
    const size_t oR = 0, oF = (sizeof(float) * img2 * IB + 255) / 256 * 256,
                 total = oF + sizeof(float2) * ft2 * IB;
    char* b = (char*)ws_get(c, WS_PREP, total, &st);
    if (!b) return st;
    float* real = (float*)(b + oR);
    cufftComplex* ft = (cufftComplex*)(b + oF);
    cudaStream_t s = c->stream;
    for (int l0 = 0; l0 < nImg; l0 += IB) {
        const int n = std::min(IB, nImg - l0);
        TG3_CUDA(cudaMemcpyAsync(ft, imgFT + 2 * ft2 * (size_t)l0, sizeof(float2) * ft2 * n,
                                 cudaMemcpyDeviceToDevice, s));
        cufftHandle hi, hf;
        if ((st = get_plan(c, N, n, &hi, true))) return st;
        if ((st = get_plan(c, N, n, &hf, false))) return st;
        if (cufftSetStream(hi, s) != CUFFT_SUCCESS || cufftExecC2R(hi, ft, real) != CUFFT_SUCCESS)
            return fail(TG3_ERR_CUDA, "cuFFT inverse transform failed");
        const size_t cnt = img2 * n;
        k_remask_real<<<(unsigned)std::min<size_t>((cnt + 255) / 256, 152 * 32), 256, 0, s>>>(
            real, N, maskRadiusPx, edgeWidth, n);
        TG3_LAUNCH_CHECK("re-mask");
        if (cufftSetStream(hf, s) != CUFFT_SUCCESS ||
            cufftExecR2C(hf, real, reinterpret_cast<cufftComplex*>(out) + ft2 * (size_t)l0) !=
                CUFFT_SUCCESS)
            return fail(TG3_ERR_CUDA, "cuFFT forward transform failed");
    }
    return TG3_OK;
}

extern "C" int tg3_ReMask(float* const* images, int nImg, int idim, float maskRadius,
                          float pixelSize, float ew)
{
    if (!images || nImg <= 0 || idim <= 0 || !(pixelSize > 0))
        return fail(TG3_ERR_ARG, "bad ReMask arguments");
    int st = TG3_OK;
    tg3_ctx* c = nullptr;
    {
        int dev = 0;
        TG3_CUDA(cudaGetDevice(&dev));
        static std::mutex mu;
        static tg3_ctx* ctxs[64] = {};
        if (dev < 0 || dev >= 64) return fail(TG3_ERR_ARG, "device ordinal out of range");
        std::lock_guard<std::mutex> lk(mu);
        if (!ctxs[dev] && (st = tg3_ctx_create(&ctxs[dev], dev))) return st;
        c = ctxs[dev];
    }
    const size_t ft2 = (size_t)idim * (idim / 2 + 1);
    const int IB = std::min(nImg, 1024);
    float* d = (float*)ws_get(c, WS_H2D, sizeof(float2) * ft2 * IB, &st);
    if (!d) return st;
    cudaStream_t s = c->stream;
    for (int l0 = 0; l0 < nImg; l0 += IB) {
        const int n = std::min(IB, nImg - l0);
        for (int i = 0; i < n; i++)
            TG3_CUDA(cudaMemcpyAsync(d + 2 * ft2 * i, images[l0 + i], sizeof(float2) * ft2,
                                     cudaMemcpyHostToDevice, s));
        if ((st = tg3_remask_d(c, d, n, idim, maskRadius / pixelSize, ew, d))) return st;
        for (int i = 0; i < n; i++)
            TG3_CUDA(cudaMemcpyAsync(images[l0 + i], d + 2 * ft2 * i, sizeof(float2) * ft2,
                                     cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaStreamSynchronize(s));
    }
    return TG3_OK;
}
