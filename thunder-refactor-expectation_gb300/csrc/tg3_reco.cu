// Reconstruction of a map from the insertion accumulators (Reconstructor::
// reconstruct, src/Reconstructor.cpp:1129-1790, 3-D, no symmetry), on the
// padded half grid vdim = N pf, coordinates (x, y, z) with x in [0, vdim/2]
// and y, z wrapped:
//   Wiener filter from the FSC (RECONSTRUCTOR_WIENER_FILTER_FSC, :1236-1262):
//     for (5 pf)^2 <= |k|^2 < (maxR pf)^2, u = rint(|k|): f = FSC[u / pf]
//     (0 past its end), clamped to [1e-3, 1 - 1e-3], f = sqrt(2 f / (1 + f))
//     when the half maps are joined; T /= f;
//   T = max(T, 1e-25); W = 1 inside maxR pf, 0 outside (:1268-1300);
//   grid correction (:1318-1460): up to 30 rounds of C = T W,
//     C = FT(iFT(C) kRL(r^2) / nf) (convoluteC, :2593-2660; kRL the MKB
//     kernel's real-space form at r = |x| / (N pf), nf = kRL(0)),
//     W /= max(|C|, 1e-6) inside maxR pf, stopping when max ||C| - 1| < 1e-2
//     or, after 10 rounds, when it failed twice in a row to fall below 0.95 x
//     the previous (checkC with RECONSTRUCTOR_CHECK_C_MAX, :2520-2590);
//     without it W = 1 / max(|T|, 1e-6) (:1463-1490);
//   V = F W inside maxR pf; the inverse transform (1 / vdim^3); the central
//   N^3 kept (VOL_EXTRACT_RL); divided by the kernel's real-space transform
//   at |x| / (pf N): j0(pi r)^2 for the trilinear kernel (TIK_RL), MKB_RL(r,
//   a pf, alpha) / MKB_RL(0, a pf, alpha) for MKB (:1700-1790).
// MKB_RL (src/Functions/Functions.cpp:128-160, order 0): with u = 2 pi a r and
// v = sqrt(|alpha^2 - u^2|), (2 pi)^1.5 a^3 / I0(alpha) I_1.5(v) / v^1.5 for
// u <= alpha, J_1.5(v) / v^1.5 beyond; the half-integer Bessel functions in
// their closed forms.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {
namespace {

// I_1.5(v) / v^1.5 and J_1.5(v) / v^1.5 (closed forms; series near 0)
__host__ __device__ double i15_over(double v)
{
    if (v < 1e-3) return (1.0 + v * v / 10.0) / (3.0 * sqrt(M_PI / 2.0));
    return sqrt(2.0 / M_PI) * (cosh(v) - sinh(v) / v) / (v * v);
}

__host__ __device__ double j15_over(double v)
{
    if (v < 1e-3) return (1.0 - v * v / 10.0) / (3.0 * sqrt(M_PI / 2.0));
    return sqrt(2.0 / M_PI) * (sin(v) / v - cos(v)) / (v * v);
}

// the modified Bessel function I0 by its power series (alpha is O(10))
__host__ __device__ double bessel_i0(double x)
{
    double s = 1.0, t = 1.0;
    const double q = x * x / 4.0;
    for (int k = 1; k < 200; k++) {
        t *= q / ((double)k * k);
        s += t;
        if (t < 1e-17 * s) break;
    }
    return s;
}

__host__ __device__ double mkb_rl(double r, double a, double alpha, double i0a)
{
    const double u = 2.0 * M_PI * a * r;
    const double w = pow(2.0 * M_PI, 1.5) * a * a * a / i0a;
    if (u <= alpha) return w * i15_over(sqrt(alpha * alpha - u * u));
    return w * j15_over(sqrt(u * u - alpha * alpha));
}

__device__ double tik_rl(double r)
{
    const double x = M_PI * r;
    const double j0 = x < 1e-8 ? 1.0 : sin(x) / x;
    return j0 * j0;
}

__device__ __forceinline__ int wrapc(int i, int n) { return i < n / 2 ? i : i - n; }

// Wiener-filtered, floored T and the initial W (1 inside the radius)
__global__ void k_reco_init(const float4* __restrict__ acc, int vdim, int nz, int pf,
                            const double* __restrict__ fsc, int nFsc, int joinHalf,
                            long long r2max, float* __restrict__ T, float* __restrict__ W)
{
    const int nx = vdim / 2 + 1;
    const size_t n = (size_t)nz * vdim * nx;
    const long long r2min = 25LL * pf * pf;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned u32 = (unsigned)idx, row = u32 / (unsigned)nx;
        const int x = (int)(u32 - row * (unsigned)nx);
        const int y = wrapc((int)(row % (unsigned)vdim), vdim);
        const int z = nz > 1 ? wrapc((int)(row / (unsigned)vdim), vdim) : 0;
        const long long q = (long long)x * x + (long long)y * y + (long long)z * z;
        double t = acc[idx].z;
        if (fsc && q >= r2min && q < r2max) {
            // rint(sqrt(q)) in FP32 is exact here: no integer q lies within
            // FP32 rounding of a half-integer radius below 2^11
            const int u = (int)rintf(sqrtf((float)q));
            double f = (u / pf >= nFsc) ? 0.0 : fsc[u / pf];
            f = fmax(1e-3, fmin(1.0 - 1e-3, f));
            if (joinHalf) f = sqrt(2.0 * f / (1.0 + f));
            t /= f;
        }
        T[idx] = (float)fmax(t, 1e-25);
        W[idx] = q < r2max ? 1.f : 0.f;
    }
}

// C = T W (real, as a complex half grid)
__global__ void k_reco_tw(const float* __restrict__ T, const float* __restrict__ W, size_t n,
                          float2* __restrict__ C)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        C[i] = make_float2(T[i] * W[i], 0.f);
}

// A radial function of the integer squared radius q, tabulated once per call
// (the kernels depend on x^2 + y^2 + z^2 only): tab[q] = scale k(sqrt(q) / s)
// with k the MKB real-space form (mkb) or j0(pi r)^2.  r2step > 0 takes the
// kernel at r^2 rounded to the nearest multiple of r2step, as a TabFunction
// of r^2 looks it up (src/TabFunction.cpp:42-45; the balancing kernel
// Reconstructor::_kernelRL is one over [0, 1] in 1e5 steps,
// src/Reconstructor.cpp:76-85).
__global__ void k_radial_table(float* __restrict__ tab, int nq, double s, int mkb, double a,
                               double alpha, double i0a, double scale, double r2step)
{
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        double r = sqrt((double)q) / s;
        if (r2step > 0) r = sqrt(rint((double)q / (s * s) / r2step) * r2step);
        tab[q] = (float)(scale * (mkb ? mkb_rl(r, a, alpha, i0a) : tik_rl(r)));
    }
}

// real-space C (after the unnormalised inverse) times kRL(r^2) / nf / vdim^3
// (the table holds kRL / nf / vdim^3)
__global__ void k_reco_kernel_rl(float* __restrict__ c, int vdim, int nz,
                                 const float* __restrict__ tab)
{
    const size_t n = (size_t)nz * vdim * vdim;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned u32 = (unsigned)idx, row = u32 / (unsigned)vdim;
        const int x = wrapc((int)(u32 - row * (unsigned)vdim), vdim);
        const int y = wrapc((int)(row % (unsigned)vdim), vdim);
        const int z = nz > 1 ? wrapc((int)(row / (unsigned)vdim), vdim) : 0;
        c[idx] *= tab[x * x + y * y + z * z];
    }
}

// W /= max(|C|, 1e-6) inside the radius; diff = max ||C| - 1| there (float
// bits compared as ints: the values are non-negative); then C <- T W for the
// next round (the inverse transform consumes C)
__global__ void k_reco_update(float2* __restrict__ C, const float* __restrict__ T, int vdim,
                              int nz, long long r2max, float* __restrict__ W,
                              unsigned* __restrict__ diffBits)
{
    const int nx = vdim / 2 + 1;
    const size_t n = (size_t)nz * vdim * nx;
    float dmax = 0.f;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned u32 = (unsigned)idx, row = u32 / (unsigned)nx;
        const int x = (int)(u32 - row * (unsigned)nx);
        const int y = wrapc((int)(row % (unsigned)vdim), vdim);
        const int z = nz > 1 ? wrapc((int)(row / (unsigned)vdim), vdim) : 0;
        const long long q = (long long)x * x + (long long)y * y + (long long)z * z;
        float w = W[idx];
        if (q < r2max) {
            const float m = sqrtf(C[idx].x * C[idx].x + C[idx].y * C[idx].y);
            w = w / fmaxf(m, 1e-6f);
            W[idx] = w;
            dmax = fmaxf(dmax, fabsf(m - 1.f));
        }
        C[idx] = make_float2(T[idx] * w, 0.f);
    }
    for (int o = 16; o; o >>= 1) dmax = fmaxf(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if ((threadIdx.x & 31) == 0) atomicMax(diffBits, __float_as_uint(dmax));
}

// without grid correction: W = 1 / max(|T|, 1e-6) inside the radius
__global__ void k_reco_w_from_t(const float* __restrict__ T, int vdim, int nz, long long r2max,
                                float* __restrict__ W)
{
    const int nx = vdim / 2 + 1;
    const size_t n = (size_t)nz * vdim * nx;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned u32 = (unsigned)idx, row = u32 / (unsigned)nx;
        const int x = (int)(u32 - row * (unsigned)nx);
        const int y = wrapc((int)(row % (unsigned)vdim), vdim);
        const int z = nz > 1 ? wrapc((int)(row / (unsigned)vdim), vdim) : 0;
        const long long q = (long long)x * x + (long long)y * y + (long long)z * z;
        if (q < r2max) W[idx] = 1.f / fmaxf(fabsf(T[idx]), 1e-6f);
    }
}

// V = F W inside the radius, 0 outside
__global__ void k_reco_fw(const float4* __restrict__ acc, const float* __restrict__ W, int vdim,
                          int nz, long long r2max, float2* __restrict__ V)
{
    const int nx = vdim / 2 + 1;
    const size_t n = (size_t)nz * vdim * nx;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const unsigned u32 = (unsigned)idx, row = u32 / (unsigned)nx;
        const int x = (int)(u32 - row * (unsigned)nx);
        const int y = wrapc((int)(row % (unsigned)vdim), vdim);
        const int z = nz > 1 ? wrapc((int)(row / (unsigned)vdim), vdim) : 0;
        const long long q = (long long)x * x + (long long)y * y + (long long)z * z;
        const float4 a = acc[idx];
        V[idx] = q < r2max ? make_float2(a.x * W[idx], a.y * W[idx]) : make_float2(0.f, 0.f);
    }
}

// the central N^3 of the padded real-space map, in centred order (index i +
// N/2 for coordinate i), divided by the kernel's real-space transform
// (the table holds the kernel's real-space transform times vdim^3)
__global__ void k_reco_extract(const float* __restrict__ pad, int vdim, int nz, int N,
                               const float* __restrict__ tab, float* __restrict__ out)
{
    const size_t n = (size_t)(nz > 1 ? N : 1) * N * N;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(idx % N) - N / 2;
        const int y = (int)((idx / N) % N) - N / 2;
        const int z = nz > 1 ? (int)(idx / ((size_t)N * N)) - N / 2 : 0;
        const int px = x < 0 ? x + vdim : x, py = y < 0 ? y + vdim : y, pz = z < 0 ? z + vdim : z;
        out[idx] = pad[((size_t)pz * vdim + py) * vdim + px] / tab[x * x + y * y + z * z];
    }
}

// accumulator <- (F, T): the sums of several contexts or ranks loaded back
__global__ void k_acc_load(const float2* __restrict__ F, const float* __restrict__ T, size_t n,
                           float4* __restrict__ acc)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        acc[i] = make_float4(F[i].x, F[i].y, T[i], 0.f);
}

struct Plan3 {
    tg3_ctx* c;
    int vdim, nz, type;
    cufftHandle h;
};
std::vector<Plan3> g_plans3;
std::mutex g_plans3Lock;

// cuFFT plan of the padded grid: vdim^3 (nz = vdim) or vdim^2 (nz = 1)
int plan3(tg3_ctx* c, int vdim, int nz, cufftType type, cufftHandle* out)
{
    std::lock_guard<std::mutex> g(g_plans3Lock);
    for (auto& p : g_plans3)
        if (p.c == c && p.vdim == vdim && p.nz == nz && p.type == (int)type) {
            *out = p.h;
            return TG3_OK;
        }
    cufftHandle h;
    const cufftResult r = nz > 1 ? cufftPlan3d(&h, vdim, vdim, vdim, type)
                                 : cufftPlan2d(&h, vdim, vdim, type);
    if (r != CUFFT_SUCCESS) return fail(TG3_ERR_CUDA, "cuFFT plan creation failed");
    g_plans3.push_back({c, vdim, nz, (int)type, h});
    *out = h;
    return TG3_OK;
}

// ---- PrepareTF: normalisation and symmetrisation of the accumulators
constexpr int kMaxSym = 64;     // symmetry elements (the icosahedral group has 59 besides E)

struct SymMats {
    double m[kMaxSym * 9];
};

// src = acc, scaled by 1 / T at the origin when normalising (allReduceT's
// RECONSTRUCTOR_NORMALISE_T_F, src/Reconstructor.cpp:2453-2480).
__global__ void k_acc_scaled_copy(const float4* __restrict__ acc, size_t n, int normalise,
                                  float4* __restrict__ src)
{
    const float sf = normalise ? 1.0f / acc[0].z : 1.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = acc[i];
        src[i] = make_float4(v.x * sf, v.y * sf, v.z * sf, 0.f);
    }
}

// Trilinear sample of the (F, T) half grid at (x, y, z), the Friedel mate
// conjugated for x < 0 (Volume::getByInterpolationFT, LINEAR_INTERP).
__device__ __forceinline__ float3 sample_ft(const float4* __restrict__ v, int vdim, float x,
                                            float y, float z)
{
    float sgn = 1.f;
    if (x < 0.f) {
        x = -x;
        y = -y;
        z = -z;
        sgn = -1.f;
    }
    const int nx = vdim / 2 + 1;
    const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
    const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
    const float fx = x - xf, fy = y - yf, fz = z - zf;
    const float wx[2] = {1.f - fx, fx}, wy[2] = {1.f - fy, fy}, wz[2] = {1.f - fz, fz};
    float3 o = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const int zz = z0 + k < 0 ? z0 + k + vdim : z0 + k;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int yy = y0 + j < 0 ? y0 + j + vdim : y0 + j;
            const float4* row = v + ((size_t)zz * vdim + yy) * nx + x0;
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const float w = wx[i] * wy[j] * wz[k];
                const float4 c = __ldg(row + i);
                o.x += c.x * w;
                o.y += c.y * w;
                o.z += c.z * w;
            }
        }
    }
    o.y *= sgn;
    return o;
}

// acc = src + sum over the symmetry elements R of src sampled at R v for
// |R v|^2 < r2 (SYMMETRIZE_FT, include/Geometry/Transformation.h:170-196),
// T floored at 1e-25 (PrepareTF's symmetrizeT).  R v and its squared norm are
// formed in FP64 in the reference's order, ((m0 i + m1 j) + m2 k) and
// (a^2 + b^2) + c^2, with every product and sum rounded on its own (no fused
// multiply-add): a voxel whose rotated image lies on the sphere |u| = r up to
// rounding is then kept or dropped as the reference keeps or drops it.
__device__ __forceinline__ double dot3_rn(const double* m, double i, double j, double k)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(m[0], i), __dmul_rn(m[1], j)), __dmul_rn(m[2], k));
}

__global__ void k_symmetrize(float4* __restrict__ acc, const float4* __restrict__ src, int vdim,
                             const SymMats mats, int nSym, double r2)
{
    const int nx = vdim / 2 + 1, half = vdim / 2;
    const size_t n = (size_t)vdim * vdim * nx;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n;
         q += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(q % nx);
        const int y = (int)((q / nx) % vdim), z = (int)(q / ((size_t)nx * vdim));
        const int j = y < half ? y : y - vdim, k = z < half ? z : z - vdim;
        float4 v = src[q];
        // a rotation keeps |v|: voxels well outside the sphere have nothing to add
        if ((double)(i * i + j * j + k * k) <= r2 + 1.0) {
            for (int s = 0; s < nSym; s++) {
                const double* m = mats.m + 9 * s;
                const double a = dot3_rn(m, i, j, k), b = dot3_rn(m + 3, i, j, k),
                             c = dot3_rn(m + 6, i, j, k);
                const double nn = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)),
                                            __dmul_rn(c, c));
                if (nn < r2) {
                    const float3 w = sample_ft(src, vdim, (float)a, (float)b, (float)c);
                    v.x += w.x;
                    v.y += w.y;
                    v.z += w.z;
                }
            }
        }
        v.z = fmaxf(v.z, 1e-25f);
        acc[q] = v;
    }
}

}  // namespace

void reco_release(tg3_ctx* c)
{
    std::lock_guard<std::mutex> g(g_plans3Lock);
    for (size_t i = 0; i < g_plans3.size();) {
        if (g_plans3[i].c == c) {
            cufftDestroy(g_plans3[i].h);
            g_plans3.erase(g_plans3.begin() + i);
        } else {
            i++;
        }
    }
}

}  // namespace tg3

using namespace tg3;

extern "C" int tg3_ctx_insert_load_d(tg3_ctx* c, const float* F, const float* T)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "no insertion accumulator (tg3_ctx_insert_begin)");
    if (!F || !T) return fail(TG3_ERR_ARG, "null device pointer");
    const int vdim = c->ins.vdim;
    const size_t n = (size_t)vdim * vdim * (vdim / 2 + 1);
    k_acc_load<<<152 * 8, 256, 0, c->stream>>>(reinterpret_cast<const float2*>(F), T, n, c->ins.acc);
    TG3_LAUNCH_CHECK("accumulator load");
    return TG3_OK;
}

namespace {

// The reconstruction chain on an accumulator acc of vdim x vdim x (vdim/2+1)
// cells (nz = vdim, 3-D) or vdim x (vdim/2+1) (nz = 1, 2-D), into out: the
// central N^3 or N^2 of the padded real-space result, N = vdim / pf.
int reconstruct_core(tg3_ctx* c, const float4* acc, int vdim, int nz, int pf, const double* fsc,
                     int nFsc, int joinHalf, int maxRadius, int gridCorr, int kernel, float a,
                     float alpha, float* vol, int* rounds)
{
    int st = TG3_OK;
    const int N = vdim / pf;
    const double cells = nz > 1 ? (double)vdim * vdim * vdim : (double)vdim * vdim;
    const size_t nh = (size_t)nz * vdim * (vdim / 2 + 1), nr = (size_t)nz * vdim * vdim;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const int nqPad = 3 * (vdim / 2) * (vdim / 2) + 1, nqBox = 3 * (N / 2) * (N / 2) + 1;
    const size_t oT = 0, oW = up(4 * nh), oC = oW + up(4 * nh), oR = oC + up(8 * nh),
                 oD = oR + up(4 * nr), oK = oD + 256, oE = oK + up(4 * (size_t)nqPad),
                 total = oE + up(4 * (size_t)nqBox);
    char* b = (char*)ws_get(c, WS_RECO, total, &st);
    if (!b) return st;
    float* T = (float*)(b + oT);
    float* W = (float*)(b + oW);
    float2* C = (float2*)(b + oC);
    float* R = (float*)(b + oR);
    unsigned* dBits = (unsigned*)(b + oD);
    float* tabK = (float*)(b + oK);
    float* tabE = (float*)(b + oE);
    cudaStream_t s = c->stream;
    const long long r2max = (long long)maxRadius * pf * maxRadius * pf;
    const int G = 152 * 8;
    k_reco_init<<<G, 256, 0, s>>>(acc, vdim, nz, pf, fsc, nFsc, joinHalf, r2max, T, W);
    TG3_LAUNCH_CHECK("reconstruction set-up");
    const double i0a = bessel_i0(alpha);
    int m = 0;
    if (gridCorr) {
        cufftHandle inv, fwd;
        if ((st = plan3(c, vdim, nz, CUFFT_C2R, &inv)) || (st = plan3(c, vdim, nz, CUFFT_R2C, &fwd)))
            return st;
        if (cufftSetStream(inv, s) != CUFFT_SUCCESS || cufftSetStream(fwd, s) != CUFFT_SUCCESS)
            return fail(TG3_ERR_CUDA, "cuFFT stream");
        const double invNf = 1.0 / mkb_rl(0.0, a, alpha, i0a);
        k_radial_table<<<(nqPad + 255) / 256, 256, 0, s>>>(tabK, nqPad, (double)N * pf, 1, a, alpha,
                                                            i0a, invNf / cells, 1.0 / 100000);
        TG3_LAUNCH_CHECK("balancing kernel table");
        float diff = 3.4e38f, prev;
        int noDecrease = 0;
        k_reco_tw<<<G, 256, 0, s>>>(T, W, nh, C);
        TG3_LAUNCH_CHECK("balancing C = T W");
        for (m = 0; m < 30; m++) {
            if (cufftExecC2R(inv, reinterpret_cast<cufftComplex*>(C), R) != CUFFT_SUCCESS)
                return fail(TG3_ERR_CUDA, "cuFFT inverse transform failed");
            k_reco_kernel_rl<<<G, 256, 0, s>>>(R, vdim, nz, tabK);
            TG3_LAUNCH_CHECK("balancing kernel product");
            if (cufftExecR2C(fwd, R, reinterpret_cast<cufftComplex*>(C)) != CUFFT_SUCCESS)
                return fail(TG3_ERR_CUDA, "cuFFT forward transform failed");
            TG3_CUDA(cudaMemsetAsync(dBits, 0, sizeof(unsigned), s));
            k_reco_update<<<G, 256, 0, s>>>(C, T, vdim, nz, r2max, W, dBits);
            TG3_LAUNCH_CHECK("balancing update");
            unsigned bits = 0;
            TG3_CUDA(cudaMemcpyAsync(&bits, dBits, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            TG3_CUDA(cudaStreamSynchronize(s));
            prev = diff;
            std::memcpy(&diff, &bits, sizeof(float));
            noDecrease = diff > prev * 0.95f ? noDecrease + 1 : 0;
            if (diff < 1e-2f || (m >= 10 && noDecrease == 2)) break;
        }
    } else {
        k_reco_w_from_t<<<G, 256, 0, s>>>(T, vdim, nz, r2max, W);
        TG3_LAUNCH_CHECK("W from T");
    }
    if (rounds) *rounds = gridCorr ? std::min(m + 1, 30) : 0;
    cufftHandle inv;
    if ((st = plan3(c, vdim, nz, CUFFT_C2R, &inv))) return st;
    if (cufftSetStream(inv, s) != CUFFT_SUCCESS) return fail(TG3_ERR_CUDA, "cuFFT stream");
    k_reco_fw<<<G, 256, 0, s>>>(acc, W, vdim, nz, r2max, C);
    TG3_LAUNCH_CHECK("F W");
    if (cufftExecC2R(inv, reinterpret_cast<cufftComplex*>(C), R) != CUFFT_SUCCESS)
        return fail(TG3_ERR_CUDA, "cuFFT inverse transform failed");
    const int mkb = kernel == TG3_KERNEL_MKB;
    const double nf = mkb ? mkb_rl(0.0, (double)a * pf, alpha, i0a) : 1.0;
    // gridding correction: the map (times the cell count after the
    // unnormalised inverse) over the kernel's real-space transform at
    // |x| / (pf N)
    k_radial_table<<<(nqBox + 255) / 256, 256, 0, s>>>(tabE, nqBox, (double)pf * N, mkb,
                                                        (double)a * pf, alpha, i0a, cells / nf, 0.0);
    TG3_LAUNCH_CHECK("gridding correction table");
    k_reco_extract<<<G, 256, 0, s>>>(R, vdim, nz, N, tabE, vol);
    TG3_LAUNCH_CHECK("extract and gridding correction");
    return TG3_OK;
}

}  // namespace

extern "C" int tg3_ctx_reconstruct_d(tg3_ctx* c, const double* fsc, int nFsc, int joinHalf,
                                     int maxRadius, int gridCorr, int kernel, float a,
                                     float alpha, float* vol, int* rounds)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "no insertion accumulator (tg3_ctx_insert_begin)");
    if (!vol || maxRadius <= 0 || (fsc && nFsc <= 0) ||
        (kernel != TG3_KERNEL_MKB && kernel != TG3_KERNEL_TRILINEAR))
        return fail(TG3_ERR_ARG, "bad reconstruction arguments");
    if ((gridCorr || kernel == TG3_KERNEL_MKB) && !(a > 0 && alpha > 0))
        return fail(TG3_ERR_ARG, "MKB parameters a and alpha must be positive");
    const int vdim = c->ins.vdim, pf = c->ins.pf;
    if (maxRadius * pf > vdim / 2) return fail(TG3_ERR_ARG, "maxRadius beyond the padded grid");
    // 32-bit voxel indices in the kernels
    if ((size_t)vdim * vdim * vdim >= (1ull << 31)) return fail(TG3_ERR_UNSUPPORTED, "padded grid above 1290^3");
    return reconstruct_core(c, c->ins.acc, vdim, vdim, pf, fsc, nFsc, joinHalf, maxRadius,
                            gridCorr, kernel, a, alpha, vol, rounds);
}

// The offsets' symmetrisation of Reconstructor::symmetrizeO (src/Reconstructor.cpp,
// under RECONSTRUCTOR_SYMMETRIZE_DURING_RECONSTRUCT): O += sum_s R_s O over
// the symmetry elements besides the identity (each R_s applied to the
// unsymmetrised O), counter *= 1 + nSym.  Host arithmetic.
extern "C" int tg3_SymmetrizeO(double* O3D, int* counter, const double* symMat, int nSym)
{
    if (!O3D || !counter || nSym < 0 || (nSym > 0 && !symMat))
        return fail(TG3_ERR_ARG, "bad symmetrizeO arguments");
    const double o[3] = {O3D[0], O3D[1], O3D[2]};
    double r[3] = {o[0], o[1], o[2]};
    for (int e = 0; e < nSym; e++) {
        const double* m = symMat + 9 * e;
        for (int i = 0; i < 3; i++) r[i] += m[3 * i] * o[0] + m[3 * i + 1] * o[1] + m[3 * i + 2] * o[2];
    }
    O3D[0] = r[0];
    O3D[1] = r[1];
    O3D[2] = r[2];
    *counter *= 1 + nSym;
    return TG3_OK;
}

// 2-D reconstruction (Reconstructor::reconstruct(Image&), MODE_2D): the same
// chain on one class's 2-D accumulators, host buffers in and out.
extern "C" int tg3_Reconstruct2D(const float* F2D, const float* T2D, int vdim, int pf,
                                 const double* fsc, int nFsc, int joinHalf, int maxRadius,
                                 int gridCorr, int kernel, float a, float alpha, float* img,
                                 int* rounds)
{
    if (!F2D || !T2D || !img || vdim < 4 || (vdim & 1) || pf < 1 || vdim % pf ||
        maxRadius <= 0 || maxRadius * pf > vdim / 2 || (fsc && nFsc <= 0) ||
        (kernel != TG3_KERNEL_MKB && kernel != TG3_KERNEL_TRILINEAR))
        return fail(TG3_ERR_ARG, "bad 2-D reconstruction arguments");
    if ((gridCorr || kernel == TG3_KERNEL_MKB) && !(a > 0 && alpha > 0))
        return fail(TG3_ERR_ARG, "MKB parameters a and alpha must be positive");
    int dev = 0;
    TG3_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static tg3_ctx* ctxs[64] = {};
    if (dev < 0 || dev >= 64) return fail(TG3_ERR_ARG, "device ordinal out of range");
    int st = TG3_OK;
    tg3_ctx* c = nullptr;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!ctxs[dev] && (st = tg3_ctx_create(&ctxs[dev], dev))) return st;
        c = ctxs[dev];
    }
    const size_t nh = (size_t)vdim * (vdim / 2 + 1);
    const int N = vdim / pf;
    const size_t oA = 0, oF = (sizeof(float4) * nh + 255) / 256 * 256,
                 oT = oF + (sizeof(float2) * nh + 255) / 256 * 256,
                 oO = oT + (sizeof(float) * nh + 255) / 256 * 256,
                 total = oO + sizeof(float) * (size_t)N * N;
    char* b = (char*)ws_get(c, WS_RECO2D, total, &st);
    if (!b) return st;
    cudaStream_t s = c->stream;
    double* dFsc = nullptr;
    if (fsc) {
        dFsc = (double*)ws_get(c, WS_MISC, sizeof(double) * nFsc, &st);
        if (!dFsc) return st;
        TG3_CUDA(cudaMemcpyAsync(dFsc, fsc, sizeof(double) * nFsc, cudaMemcpyHostToDevice, s));
    }
    TG3_CUDA(cudaMemcpyAsync(b + oF, F2D, sizeof(float2) * nh, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oT, T2D, sizeof(float) * nh, cudaMemcpyHostToDevice, s));
    float4* acc = (float4*)(b + oA);
    k_acc_load<<<152 * 2, 256, 0, s>>>((const float2*)(b + oF), (const float*)(b + oT), nh, acc);
    TG3_LAUNCH_CHECK("2-D accumulator load");
    if ((st = reconstruct_core(c, acc, vdim, 1, pf, dFsc, nFsc, joinHalf, maxRadius, gridCorr,
                               kernel, a, alpha, (float*)(b + oO), rounds)))
        return st;
    TG3_CUDA(cudaMemcpyAsync(img, b + oO, sizeof(float) * (size_t)N * N, cudaMemcpyDeviceToHost,
                             s));
    return tg3_ctx_sync(c);
}

extern "C" int tg3_ctx_prepare_tf_d(tg3_ctx* c, const double* symMat, int nSym, int maxRadius,
                                    int normalise)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "no insertion accumulator (tg3_ctx_insert_begin)");
    if (nSym < 0 || nSym > kMaxSym || (nSym > 0 && !symMat))
        return fail(TG3_ERR_ARG, "symmetry elements: 0 to 64 matrices");
    const int vdim = c->ins.vdim, pf = c->ins.pf;
    const double r = (double)maxRadius * pf + 1.0;
    if (maxRadius <= 0 || r + 1.0 > vdim / 2)
        return fail(TG3_ERR_ARG, "maxRadius x pf + 2 must not exceed vdim / 2");
    SymMats mats;
    for (int i = 0; i < 9 * nSym; i++) mats.m[i] = symMat[i];
    const size_t n = (size_t)vdim * vdim * (vdim / 2 + 1);
    float4* src = (float4*)ws_get(c, WS_RECO, sizeof(float4) * n, &st);
    if (!src) return st;
    cudaStream_t s = c->stream;
    k_acc_scaled_copy<<<152 * 8, 256, 0, s>>>(c->ins.acc, n, normalise, src);
    TG3_LAUNCH_CHECK("accumulator copy");
    k_symmetrize<<<152 * 16, 256, 0, s>>>(c->ins.acc, src, vdim, mats, nSym, r * r);
    TG3_LAUNCH_CHECK("symmetrisation");
    return TG3_OK;
}

extern "C" int tg3_PrepareTF(float* F3D, float* T3D, int vdim, const double* symMat, int nSym,
                             int maxRadius, int pf)
{
    if (!F3D || !T3D || vdim < 4 || (vdim & 1) || pf < 1)
        return fail(TG3_ERR_ARG, "bad PrepareTF arguments");
    int dev = 0;
    TG3_CUDA(cudaGetDevice(&dev));
    static std::mutex mu;
    static tg3_ctx* ctxs[64] = {};
    if (dev < 0 || dev >= 64) return fail(TG3_ERR_ARG, "device ordinal out of range");
    tg3_ctx* c = nullptr;
    int st = TG3_OK;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!ctxs[dev] && (st = tg3_ctx_create(&ctxs[dev], dev))) return st;
        c = ctxs[dev];
    }
    if ((st = tg3_ctx_insert_begin(c, vdim, pf))) return st;
    const size_t n = (size_t)vdim * vdim * (vdim / 2 + 1);
    float* d = (float*)ws_get(c, WS_D2H, sizeof(float) * 3 * n, &st);
    if (!d) return st;
    cudaStream_t s = c->stream;
    TG3_CUDA(cudaMemcpyAsync(d, F3D, sizeof(float) * 2 * n, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(d + 2 * n, T3D, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    if ((st = tg3_ctx_insert_load_d(c, d, d + 2 * n))) return st;
    if ((st = tg3_ctx_prepare_tf_d(c, symMat, nSym, maxRadius, 1))) return st;
    if ((st = tg3_ctx_insert_read_d(c, d, d + 2 * n, 0))) return st;
    TG3_CUDA(cudaMemcpyAsync(F3D, d, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(T3D, d + 2 * n, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaStreamSynchronize(s));
    return TG3_OK;
}
