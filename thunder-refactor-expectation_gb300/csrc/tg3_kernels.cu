// tg3_kernels.cu -- the plain (FP32) E-step and insertion kernels for sm_103a.
//
// Data layout in HBM (all particle-major):
//   projection volume  : 64-byte corner blocks (see k_volume_blocks), all
//                        eight corners of a trilinear sample in one half
//                        cache line, read by two lanes with one 256-bit load
//                        each, placed in 32^3-voxel cubes (brick_index);
//   projections P      : [row][Kp] floats, a complex row padded with zeros to
//                        Kp floats (Kp a multiple of 64);
//   shifted data A''   : [particle][translation][Kp] floats, the complex
//                        sigRcp * ctf * X * exp(+2 pi i k.t / N);
//   log-likelihoods D  : [particle][rotation][translation] floats, without the
//                        per-particle constant sum sigRcp |X|^2;
//   insertion volume   : float4 [vdim][vdim][nx] of (F.re, F.im, T, 0), one
//                        16-byte atomic per voxel update.
#include <algorithm>

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "tg3_internal.cuh"

namespace tg3 {

namespace {

// Store one complex value at element pair p of row `row` (pitch ldo
// elements): as two floats, or -- when splitLo != 0 -- as the bf16 pair
// hi = bf16(v) in the plane at `out` and lo = bf16(v - hi) in the plane
// splitLo elements further on.
__device__ __forceinline__ void store_pair(float* out, long long splitLo, size_t row, int ldo,
                                           int p, float a, float b)
{
    if (splitLo == 0) {
        reinterpret_cast<float2*>(out + row * ldo)[p] = make_float2(a, b);
        return;
    }
    __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(out);
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    reinterpret_cast<__nv_bfloat162*>(hi + row * ldo)[p] = h;
    reinterpret_cast<__nv_bfloat162*>(hi + splitLo + row * ldo)[p] = l;
}

// Lane-pair form of store_pair: both lanes of a pair hold (a, b); lane half
// h stores its share -- the real (h = 0) or imaginary (h = 1) float, or the
// hi (h = 0) or lo (h = 1) bf16 pair -- so a warp's stores are contiguous.
__device__ __forceinline__ void store_pair_half(float* out, long long splitLo, size_t row, int ldo,
                                                int p, int h, float a, float b)
{
    if (splitLo == 0) {
        out[row * ldo + 2 * (size_t)p + h] = h ? b : a;
        return;
    }
    __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(out);
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    if (h) {
        const float2 hf = __bfloat1622float2(v);
        v = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    }
    reinterpret_cast<__nv_bfloat162*>(hi + (h ? splitLo : 0) + row * ldo)[p] = v;
}

__device__ __forceinline__ float warp_sum(float v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_max(float v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum (double) through shared scratch of >= 32 doubles.
__device__ double block_sum_d(double v, double* scratch)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
    v = warp_sum_d(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    double r = 0;
    if (wid == 0) {
        r = lane < nw ? scratch[lane] : 0.0;
        r = warp_sum_d(r);
        if (lane == 0) scratch[0] = r;
    }
    __syncthreads();
    r = scratch[0];
    __syncthreads();
    return r;
}

// Quaternion -> row-major rotation matrix, R = I + 2 w A + 2 A^2
// (rotate3D, src/Geometry/Euler.cpp:181-189).
__device__ __forceinline__ void quat_to_mat(const double* q, double* m)
{
    const double A[3][3] = {{0, -q[3], q[2]}, {q[3], 0, -q[1]}, {-q[2], q[1], 0}};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double aa = (2 * A[i][0]) * A[0][j] + (2 * A[i][1]) * A[1][j]
                      + (2 * A[i][2]) * A[2][j];
            m[3 * i + j] = ((i == j ? 1.0 : 0.0) + (2 * q[0]) * A[i][j]) + aa;
        }
}

// ------------------------------------------------------------------------
__global__ void k_rotmat(const double* __restrict__ quat, int n, double* __restrict__ mat)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    double q[4] = {quat[4 * r], quat[4 * r + 1], quat[4 * r + 2], quat[4 * r + 3]};
    quat_to_mat(q, mat + 9 * (size_t)r);
}

// Phase-shift bank S[t][p] = exp(-2 pi i (iCol tx + iRow ty) / N)
// (translate, src/Image/ImageFunctions.cpp:233-252).
__global__ void k_translate(const double* __restrict__ trans, int nT, int idim,
                            const int* __restrict__ iCol, const int* __restrict__ iRow,
                            int K, float2* __restrict__ out, int ldo2)
{
    const int t = blockIdx.y;
    const float tx = (float)trans[2 * t], ty = (float)trans[2 * t + 1];
    const float invN = 1.0f / (float)idim;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldo2; p += gridDim.x * blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (p < K) {
            float f = ((float)iCol[p] * tx + (float)iRow[p] * ty) * invN;
            float s, c;
            sincospif(2.0f * f, &s, &c);
            v = make_float2(c, -s);
        }
        out[(size_t)t * ldo2 + p] = v;
    }
}

// CTF at the selected pixels (CTF(RFLOAT*, ...), src/CTF.cpp:98-145).
__global__ void k_ctf(const float* __restrict__ attr, int nImg, float px, int idim,
                      const int* __restrict__ iCol, const int* __restrict__ iRow,
                      int K, float* __restrict__ out)
{
    const int l = blockIdx.x;
    const float* a = attr + 7 * (size_t)l;
    const float V = a[0], dU = a[1], dV = a[2], th = a[3], Cs = a[4], A = a[5], ps = a[6];
    const float lambda = 12.2643247f / sqrtf(V * (1 + V * 0.978466e-6f));
    const float w1 = sqrtf(1 - A * A), w2 = A;
    const float K1 = CUDART_PI_F * lambda;
    const float K2 = (CUDART_PI_F / 2) * Cs * lambda * lambda * lambda;
    const float inv = 1.0f / (px * (float)idim);
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        float u = hypotf((float)iCol[p] * inv, (float)iRow[p] * inv);
        float ang = atan2f((float)iRow[p], (float)iCol[p]) - th;
        float dfc = -(dU + dV + (dU - dV) * cosf(2 * ang)) / 2;
        float u2 = u * u;
        float ki = K1 * dfc * u2 + K2 * u2 * u2 - ps;
        out[(size_t)l * K + p] = -w1 * sinf(ki) + w2 * cosf(ki);
    }
}

// Placement of voxel (z, y, x)'s corner block: the volume is cut into
// cubes of 32^3 voxels (32768 blocks = 2 MB, one large page each, cubes in
// z, y, x order), each cube into 4^3 bricks of 8^3 voxels, voxels x-fastest
// within a brick.  A projection's samples within one pixel band then touch a
// few hundred pages instead of one page per z plane of the band, which in
// the plain [z][y][x] order left the gather translation-bound.
__device__ __forceinline__ size_t brick_index(int x, int y, int z, int nxc, int nyc)
{
    const size_t cube = ((size_t)(z >> 5) * nyc + (y >> 5)) * nxc + (x >> 5);
    const int brick = (((z >> 3) & 3) * 4 + ((y >> 3) & 3)) * 4 + ((x >> 3) & 3);
    const int v = ((z & 7) * 8 + (y & 7)) * 8 + (x & 7);
    return (cube * 64 + brick) * 512 + v;
}


// Corner-block content: the 64-byte element of voxel (z, y, x) holds, for
// slab z then slab z + 1, V[.][y][x], V[.][y][x+1], V[.][y+1][x],
// V[.][y+1][x+1] (rows and slabs taken modulo vdim, the wrap of
// Volume::iFTHalf; x + 1 past the stored half reads zero).  A trilinear
// sample then reads one aligned half cache line.
__global__ void k_volume_blocks(const float2* __restrict__ vol, int vdim,
                                float4* __restrict__ blocks)
{
    const int nx = vdim / 2 + 1;
    const int nxc = cubes_x(vdim), nyc = cubes_yz(vdim);
    const size_t n = (size_t)vdim * vdim * nx;
    const float2 zero = make_float2(0.f, 0.f);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx);
        const int y = (int)((i / nx) % vdim);
        const int z = (int)(i / ((size_t)nx * vdim));
        const size_t d = brick_index(x, y, z, nxc, nyc);
        const int y1 = y + 1 == vdim ? 0 : y + 1;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int zz = k == 0 ? z : (z + 1 == vdim ? 0 : z + 1);
            const size_t i0 = ((size_t)zz * vdim + y) * nx + x;
            const size_t i1 = ((size_t)zz * vdim + y1) * nx + x;
            const float2 a = vol[i0], b = (x + 1 < nx) ? vol[i0 + 1] : zero;
            const float2 c = vol[i1], dd = (x + 1 < nx) ? vol[i1 + 1] : zero;
            blocks[4 * d + 2 * k] = make_float4(a.x, a.y, b.x, b.y);
            blocks[4 * d + 2 * k + 1] = make_float4(c.x, c.y, dd.x, dd.y);
        }
    }
}

// ------------------------------------------------------------------------
// Fourier-slice extraction: P[row][p] = trilinear(V, R_row (iCol pf, iRow pf,
// 0)), Friedel-mirrored when x < 0 (Projector::project,
// src/Projector.cpp:356-374; Volume::getByInterpolationFT,
// src/Image/Volume.cpp:308-332).
//
// Work order.  A CTA takes one pixel chunk (kProjChunk consecutive pixels) of
// one particle for a group of kProjG of its rotations, and consecutive CTAs
// take the rotation groups of the same chunk.  The CTAs resident at any time
// therefore sweep one narrow band of pixels through all of a particle's
// rotations: the volume blocks that band touches (a few MB) stay in L2 while
// every rotation that reuses them runs, instead of the particle's whole
// footprint (about 160 MB at box 256) streaming from HBM once per reuse.
//
// A lane pair serves one pixel: lane half h reads slab z0 + h of the pixel's
// 64-byte corner block (one 256-bit load) and the two partial sums meet
// through one shuffle.  Each pair carries kProjU pixels of the chunk, whose
// indices and norm weights are loaded once for all the CTA's rotations.
//
// With nrmPart != null, nrmPart[row * nChunks + chunk] receives the chunk's
// share of sum_p sigRcp ctf^2 |P|^2 (k_norm_reduce sums the chunks).
__global__ void __launch_bounds__(256, 4)
k_project(float4* const* __restrict__ volTable, const int* __restrict__ cls,
          const float4* __restrict__ vol0, int vdim, int pf, const float* __restrict__ mf,
          int rowsPerParticle, int nGroups, int nChunks, const int* __restrict__ iCol,
          const int* __restrict__ iRow, int K, float* __restrict__ out, int ldo,
          const float* __restrict__ sigRcp, const float* __restrict__ ctf,
          float* __restrict__ nrmPart, int* __restrict__ flag, long long splitLo)
{
    __shared__ float m[kProjG][9];
    __shared__ float red[kProjG][8];
    const int g = blockIdx.x % nGroups;
    const int chunk = (blockIdx.x / nGroups) % nChunks;
    const int l = blockIdx.x / (nGroups * nChunks);
    const int r0 = g * kProjG;
    const int nRot = min(kProjG, rowsPerParticle - r0);
    const size_t row0 = (size_t)l * rowsPerParticle + r0;
    // brick_index split into per-axis terms: tx[x] + ty[y + vdim/2] +
    // tz[z + vdim/2], the y and z tables absorbing the wrap of negative rows
    extern __shared__ int tab[];
    const int half = vdim / 2;
    int* tx = tab;
    int* ty = tab + vdim / 2 + 1;
    int* tz = ty + vdim;
    fill_brick_tables(vdim, tx, ty, tz);
    if (threadIdx.x < 9 * nRot) m[threadIdx.x / 9][threadIdx.x % 9] = mf[9 * row0 + threadIdx.x];
    __syncthreads();
    const int nOut = ldo / 2;
    const int h = threadIdx.x & 1;
    const int npairs = blockDim.x >> 1;
    const int pBase = chunk * kProjChunk + (threadIdx.x >> 5) * 16 + ((threadIdx.x & 31) >> 1);
    const float4* __restrict__ vol = vol0;
    if (volTable) {
        const int k = cls ? cls[l] : 0;
        vol = (k >= 0 && k < kMaxClasses) ? volTable[k] : nullptr;
        if (!vol) {
            // unknown class: record it, leave the rows' chunk zero and skip sampling
            if (threadIdx.x == 0 && flag) atomicOr(flag, 8);
            for (int i = 0; i < nRot; i++)
#pragma unroll
                for (int u = 0; u < kProjU; u++) {
                    const int p = pBase + u * npairs;
                    if (p < nOut) store_pair_half(out, splitLo, row0 + i, ldo, p, h, 0.f, 0.f);
                }
            if (nrmPart && threadIdx.x < nRot) nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = 0.f;
            return;
        }
    }
    const float fpf = (float)pf;
    const float* sg = sigRcp ? sigRcp + (size_t)l * K : nullptr;
    const float* cf = ctf ? ctf + (size_t)l * K : nullptr;
    // the chunk's pixels: coordinates and norm weights, shared by all rotations
    float pa[kProjU], pb[kProjU], w2[kProjU];
#pragma unroll
    for (int u = 0; u < kProjU; u++) {
        const int p = pBase + u * npairs;
        const int q = p < K ? p : 0;
        pa[u] = (float)iCol[q] * fpf;
        pb[u] = (float)iRow[q] * fpf;
        w2[u] = (nrmPart && p < K) ? sg[q] * cf[q] * cf[q] : 0.f;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll 1
    for (int i = 0; i < nRot; i++) {   // nRot is uniform across the CTA
        const float* mm = m[i];
        float acc = 0.f;
        float fw[kProjU][3];
        bool cj[kProjU];
        const float4* e[kProjU];
#pragma unroll
        for (int u = 0; u < kProjU; u++) {
            float x = mm[0] * pa[u] + mm[1] * pb[u];
            float y = mm[3] * pa[u] + mm[4] * pb[u];
            float z = mm[6] * pa[u] + mm[7] * pb[u];
            cj[u] = x < 0.f;
            if (cj[u]) { x = -x; y = -y; z = -z; }
            const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
            const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
            fw[u][0] = x - xf;
            fw[u][1] = y - yf;
            fw[u][2] = z - zf;
            const unsigned blk = (unsigned)(tx[x0] + ty[y0 + half] + tz[z0 + half]);
            e[u] = vol + 4 * (size_t)blk + 2 * h;
        }
        float4 c[kProjU][2];
#pragma unroll
        for (int u = 0; u < kProjU; u++)
            asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                : "=f"(c[u][0].x), "=f"(c[u][0].y), "=f"(c[u][0].z), "=f"(c[u][0].w),
                  "=f"(c[u][1].x), "=f"(c[u][1].y), "=f"(c[u][1].z), "=f"(c[u][1].w)
                : "l"(e[u]));
#pragma unroll
        for (int u = 0; u < kProjU; u++) {
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
            const int p = pBase + u * npairs;
            if (p < nOut) {
                if (p < K) {
                    if (cj[u]) im = -im;
                    store_pair_half(out, splitLo, row0 + i, ldo, p, h, re, im);
                    if (h == 0) acc = fmaf(w2[u], re * re + im * im, acc);
                } else {
                    store_pair_half(out, splitLo, row0 + i, ldo, p, h, 0.f, 0.f);
                }
            }
        }
        // the warp's share of this rotation's norm, in a fixed order
        if (nrmPart) {
            acc = warp_sum(acc);
            if (lane == 0) red[i][wid] = acc;
        }
    }
    if (nrmPart) {
        __syncthreads();
        if (threadIdx.x < nRot) {
            float s = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[threadIdx.x][w];
            nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = s;
        }
    }
}

// The same extraction with one lane per pixel (form 1).  A lane reads both
// slabs of its pixel's corner block (two 256-bit loads) and forms the sample
// alone, so the coordinates, the block address and the fractions are
// computed once per sample instead of once per lane of a pair, and no
// shuffle joins the halves.  The slab sums are formed in the pair form's
// order (slab z0's four corners, slab z0 + 1's, then their sum).  Pixels:
// p = chunk kProjChunk + u blockDim + threadIdx, u < kProjChunk / blockDim.
// A warp's 32 pixels are consecutive, so its hi and lo (or FP32) stores are
// 128-byte (256-byte) runs.
// kArith forms the block index from the coordinates with integer
// arithmetic instead of the per-axis shared-memory tables: lanes of a warp
// look up scattered table entries, and those lookups share the L1 data pipe
// with the corner-block loads.
constexpr int kLaneU = kProjChunk / 256;
template <bool kArith>
__global__ void __launch_bounds__(256, 4)
k_project_lane(float4* const* __restrict__ volTable, const int* __restrict__ cls,
               const float4* __restrict__ vol0, int vdim, int pf, const float* __restrict__ mf,
               int rowsPerParticle, int nGroups, int nChunks, const int* __restrict__ iCol,
               const int* __restrict__ iRow, int K, float* __restrict__ out, int ldo,
               const float* __restrict__ sigRcp, const float* __restrict__ ctf,
               float* __restrict__ nrmPart, int* __restrict__ flag, long long splitLo)
{
    __shared__ float m[kProjG][9];
    __shared__ float red[kProjG][8];
    const int g = blockIdx.x % nGroups;
    const int chunk = (blockIdx.x / nGroups) % nChunks;
    const int l = blockIdx.x / (nGroups * nChunks);
    const int r0 = g * kProjG;
    const int nRot = min(kProjG, rowsPerParticle - r0);
    const size_t row0 = (size_t)l * rowsPerParticle + r0;
    extern __shared__ int tab[];
    const int half = vdim / 2;
    const int nxc = cubes_x(vdim), nyc = cubes_yz(vdim);
    int* tx = tab;
    int* ty = tab + vdim / 2 + 1;
    int* tz = ty + vdim;
    if (!kArith) fill_brick_tables(vdim, tx, ty, tz);
    if (threadIdx.x < 9 * nRot) m[threadIdx.x / 9][threadIdx.x % 9] = mf[9 * row0 + threadIdx.x];
    __syncthreads();
    const int nOut = ldo / 2;
    const int pBase = chunk * kProjChunk + threadIdx.x;
    __nv_bfloat162* hiPlane = reinterpret_cast<__nv_bfloat162*>(out);
    __nv_bfloat162* loPlane = reinterpret_cast<__nv_bfloat162*>(
        reinterpret_cast<__nv_bfloat16*>(out) + splitLo);
    auto store = [&](size_t row, int p, float re, float im) {
        if (splitLo == 0) {
            reinterpret_cast<float2*>(out + row * ldo)[p] = make_float2(re, im);
        } else {
            const __nv_bfloat162 v = __floats2bfloat162_rn(re, im);
            const float2 hf = __bfloat1622float2(v);
            hiPlane[row * nOut + p] = v;
            loPlane[row * nOut + p] = __floats2bfloat162_rn(re - hf.x, im - hf.y);
        }
    };
    const float4* __restrict__ vol = vol0;
    if (volTable) {
        const int k = cls ? cls[l] : 0;
        vol = (k >= 0 && k < kMaxClasses) ? volTable[k] : nullptr;
        if (!vol) {
            // unknown class: record it, leave the rows' chunk zero and skip sampling
            if (threadIdx.x == 0 && flag) atomicOr(flag, 8);
            for (int i = 0; i < nRot; i++)
#pragma unroll
                for (int u = 0; u < kLaneU; u++) {
                    const int p = pBase + u * 256;
                    if (p < nOut) store(row0 + i, p, 0.f, 0.f);
                }
            if (nrmPart && threadIdx.x < nRot) nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = 0.f;
            return;
        }
    }
    const float fpf = (float)pf;
    const float* sg = sigRcp ? sigRcp + (size_t)l * K : nullptr;
    const float* cf = ctf ? ctf + (size_t)l * K : nullptr;
    float pa[kLaneU], pb[kLaneU], w2[kLaneU];
#pragma unroll
    for (int u = 0; u < kLaneU; u++) {
        const int p = pBase + u * 256;
        const int q = p < K ? p : 0;
        pa[u] = (float)iCol[q] * fpf;
        pb[u] = (float)iRow[q] * fpf;
        w2[u] = (nrmPart && p < K) ? sg[q] * cf[q] * cf[q] : 0.f;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll 1
    for (int i = 0; i < nRot; i++) {   // nRot is uniform across the CTA
        const float* mm = m[i];
        float acc = 0.f;
        float fw[kLaneU][3];
        bool cj[kLaneU];
        const float4* e[kLaneU];
#pragma unroll
        for (int u = 0; u < kLaneU; u++) {
            float x = mm[0] * pa[u] + mm[1] * pb[u];
            float y = mm[3] * pa[u] + mm[4] * pb[u];
            float z = mm[6] * pa[u] + mm[7] * pb[u];
            cj[u] = x < 0.f;
            if (cj[u]) { x = -x; y = -y; z = -z; }
            const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
            const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
            fw[u][0] = x - xf;
            fw[u][1] = y - yf;
            fw[u][2] = z - zf;
            unsigned blk;
            if (kArith) {
                // brick_index with the rows' and slabs' wrap of negative indices
                const int yy = y0 < 0 ? y0 + vdim : y0;
                const int zz = z0 < 0 ? z0 + vdim : z0;
                blk = (unsigned)((((zz >> 5) * nyc + (yy >> 5)) * nxc + (x0 >> 5)) * 32768
                                 + ((((zz >> 3) & 3) * 4 + ((yy >> 3) & 3)) * 4 + ((x0 >> 3) & 3)) * 512
                                 + ((zz & 7) * 8 + (yy & 7)) * 8 + (x0 & 7));
            } else {
                blk = (unsigned)(tx[x0] + ty[y0 + half] + tz[z0 + half]);
            }
            e[u] = vol + 4 * (size_t)blk;
        }
        float4 c[kLaneU][4];
#pragma unroll
        for (int u = 0; u < kLaneU; u++)
#pragma unroll
            for (int k = 0; k < 2; k++)
                asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                    : "=f"(c[u][2 * k].x), "=f"(c[u][2 * k].y), "=f"(c[u][2 * k].z),
                      "=f"(c[u][2 * k].w), "=f"(c[u][2 * k + 1].x), "=f"(c[u][2 * k + 1].y),
                      "=f"(c[u][2 * k + 1].z), "=f"(c[u][2 * k + 1].w)
                    : "l"(e[u] + 2 * k));
#pragma unroll
        for (int u = 0; u < kLaneU; u++) {
            const float fx = fw[u][0], fy = fw[u][1], fz = fw[u][2];
            const float wx0 = 1.f - fx, wx1 = fx;
            float sr[2], si[2];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const float wz = k ? fz : 1.f - fz;
                const float wy0 = (1.f - fy) * wz, wy1 = fy * wz;
                const float4 a = c[u][2 * k], b = c[u][2 * k + 1];
                float re = a.x * (wx0 * wy0) + a.z * (wx1 * wy0);
                float im = a.y * (wx0 * wy0) + a.w * (wx1 * wy0);
                re += b.x * (wx0 * wy1) + b.z * (wx1 * wy1);
                im += b.y * (wx0 * wy1) + b.w * (wx1 * wy1);
                sr[k] = re;
                si[k] = im;
            }
            float re = sr[0] + sr[1];
            float im = si[0] + si[1];
            const int p = pBase + u * 256;
            if (p < nOut) {
                if (p < K) {
                    if (cj[u]) im = -im;
                    store(row0 + i, p, re, im);
                    acc = fmaf(w2[u], re * re + im * im, acc);
                } else {
                    store(row0 + i, p, 0.f, 0.f);
                }
            }
        }
        if (nrmPart) {
            acc = warp_sum(acc);
            if (lane == 0) red[i][wid] = acc;
        }
    }
    if (nrmPart) {
        __syncthreads();
        if (threadIdx.x < nRot) {
            float s = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[threadIdx.x][w];
            nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = s;
        }
    }
}

// Lane pairs that share loads but not the coordinate work (forms 3 and 4).
// Every lane finds the block index and fractions of its own pixel (as in the
// one-lane form: once per sample), then a pair swaps them by one shuffle
// each.  The pair's two loads read pixel A's block (lane 0 slab z0, lane 1
// slab z0 + 1) and then pixel B's, so every load instruction takes whole
// 64-byte blocks, one L1 wavefront per pixel as in the lane-pair form.
// Each lane forms its slab's share of both pixels; lane 0 keeps A and lane 1
// B, the other share arriving by shuffle (slab z0's share plus slab z0 + 1's,
// the pair form's sum).  (Recomputing the partner's fractions from its
// coordinates instead of receiving them by three shuffles measured slower:
// 8.99 against 8.56 ms per 128 particles at box 256.)
template <bool kArith, int G>
__global__ void __launch_bounds__(256, 4)
k_project_xchg(float4* const* __restrict__ volTable, const int* __restrict__ cls,
               const float4* __restrict__ vol0, int vdim, int pf, const float* __restrict__ mf,
               int rowsPerParticle, int nGroups, int nChunks, const int* __restrict__ iCol,
               const int* __restrict__ iRow, int K, float* __restrict__ out, int ldo,
               const float* __restrict__ sigRcp, const float* __restrict__ ctf,
               float* __restrict__ nrmPart, int* __restrict__ flag, long long splitLo)
{
    __shared__ float m[G][9];
    __shared__ float red[G][8];
    const int g = blockIdx.x % nGroups;
    const int chunk = (blockIdx.x / nGroups) % nChunks;
    const int l = blockIdx.x / (nGroups * nChunks);
    const int r0 = g * G;
    const int nRot = min(G, rowsPerParticle - r0);
    const size_t row0 = (size_t)l * rowsPerParticle + r0;
    extern __shared__ int tab[];
    const int half = vdim / 2;
    const int nxc = cubes_x(vdim), nyc = cubes_yz(vdim);
    int* tx = tab;
    int* ty = tab + vdim / 2 + 1;
    int* tz = ty + vdim;
    if (!kArith) fill_brick_tables(vdim, tx, ty, tz);
    if (threadIdx.x < 9 * nRot) m[threadIdx.x / 9][threadIdx.x % 9] = mf[9 * row0 + threadIdx.x];
    __syncthreads();
    const int nOut = ldo / 2;
    const int h = threadIdx.x & 1;
    const int pBase = chunk * kProjChunk + threadIdx.x;
    __nv_bfloat162* hiPlane = reinterpret_cast<__nv_bfloat162*>(out);
    __nv_bfloat162* loPlane = reinterpret_cast<__nv_bfloat162*>(
        reinterpret_cast<__nv_bfloat16*>(out) + splitLo);
    auto store = [&](size_t row, int p, float re, float im) {
        if (splitLo == 0) {
            reinterpret_cast<float2*>(out + row * ldo)[p] = make_float2(re, im);
        } else {
            const __nv_bfloat162 v = __floats2bfloat162_rn(re, im);
            const float2 hf = __bfloat1622float2(v);
            hiPlane[row * nOut + p] = v;
            loPlane[row * nOut + p] = __floats2bfloat162_rn(re - hf.x, im - hf.y);
        }
    };
    const float4* __restrict__ vol = vol0;
    if (volTable) {
        const int k = cls ? cls[l] : 0;
        vol = (k >= 0 && k < kMaxClasses) ? volTable[k] : nullptr;
        if (!vol) {
            // unknown class: record it, leave the rows' chunk zero and skip sampling
            if (threadIdx.x == 0 && flag) atomicOr(flag, 8);
            for (int i = 0; i < nRot; i++)
#pragma unroll
                for (int u = 0; u < kLaneU; u++) {
                    const int p = pBase + u * 256;
                    if (p < nOut) store(row0 + i, p, 0.f, 0.f);
                }
            if (nrmPart && threadIdx.x < nRot) nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = 0.f;
            return;
        }
    }
    const float fpf = (float)pf;
    const float* sg = sigRcp ? sigRcp + (size_t)l * K : nullptr;
    const float* cf = ctf ? ctf + (size_t)l * K : nullptr;
    float pa[kLaneU], pb[kLaneU], w2[kLaneU];
#pragma unroll
    for (int u = 0; u < kLaneU; u++) {
        const int p = pBase + u * 256;
        const int q = p < K ? p : 0;
        pa[u] = (float)iCol[q] * fpf;
        pb[u] = (float)iRow[q] * fpf;
        w2[u] = (nrmPart && p < K) ? sg[q] * cf[q] * cf[q] : 0.f;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll 1
    for (int i = 0; i < nRot; i++) {   // nRot is uniform across the CTA
        const float* mm = m[i];
        float acc = 0.f;
        float fo[kLaneU][3], fp[kLaneU][3];   // own and partner fractions
        bool cj[kLaneU];
        unsigned bo[kLaneU], bp[kLaneU];      // own and partner block index
#pragma unroll
        for (int u = 0; u < kLaneU; u++) {
            float x = mm[0] * pa[u] + mm[1] * pb[u];
            float y = mm[3] * pa[u] + mm[4] * pb[u];
            float z = mm[6] * pa[u] + mm[7] * pb[u];
            cj[u] = x < 0.f;
            if (cj[u]) { x = -x; y = -y; z = -z; }
            const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
            const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
            fo[u][0] = x - xf;
            fo[u][1] = y - yf;
            fo[u][2] = z - zf;
            if (kArith) {
                const int yy = y0 < 0 ? y0 + vdim : y0;
                const int zz = z0 < 0 ? z0 + vdim : z0;
                bo[u] = (unsigned)((((zz >> 5) * nyc + (yy >> 5)) * nxc + (x0 >> 5)) * 32768
                                   + ((((zz >> 3) & 3) * 4 + ((yy >> 3) & 3)) * 4 + ((x0 >> 3) & 3)) * 512
                                   + ((zz & 7) * 8 + (yy & 7)) * 8 + (x0 & 7));
            } else {
                bo[u] = (unsigned)(tx[x0] + ty[y0 + half] + tz[z0 + half]);
            }
            bp[u] = __shfl_xor_sync(0xffffffffu, bo[u], 1);
#pragma unroll
            for (int k = 0; k < 3; k++) fp[u][k] = __shfl_xor_sync(0xffffffffu, fo[u][k], 1);
        }
        // slab h of pixel A (the even lane's) then of pixel B (the odd lane's)
        float4 c[kLaneU][4];
#pragma unroll
        for (int u = 0; u < kLaneU; u++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const unsigned b = (k == 0) == (h == 0) ? bo[u] : bp[u];
                const float4* e = vol + 4 * (size_t)b + 2 * h;
                asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                    : "=f"(c[u][2 * k].x), "=f"(c[u][2 * k].y), "=f"(c[u][2 * k].z),
                      "=f"(c[u][2 * k].w), "=f"(c[u][2 * k + 1].x), "=f"(c[u][2 * k + 1].y),
                      "=f"(c[u][2 * k + 1].z), "=f"(c[u][2 * k + 1].w)
                    : "l"(e));
            }
#pragma unroll
        for (int u = 0; u < kLaneU; u++) {
            float sr[2], si[2];
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const bool own = (k == 0) == (h == 0);
                const float fx = own ? fo[u][0] : fp[u][0];
                const float fy = own ? fo[u][1] : fp[u][1];
                const float fz = own ? fo[u][2] : fp[u][2];
                const float wz = h ? fz : 1.f - fz;
                const float wx0 = 1.f - fx, wx1 = fx;
                const float wy0 = (1.f - fy) * wz, wy1 = fy * wz;
                const float4 a = c[u][2 * k], b = c[u][2 * k + 1];
                float re = a.x * (wx0 * wy0) + a.z * (wx1 * wy0);
                float im = a.y * (wx0 * wy0) + a.w * (wx1 * wy0);
                re += b.x * (wx0 * wy1) + b.z * (wx1 * wy1);
                im += b.y * (wx0 * wy1) + b.w * (wx1 * wy1);
                sr[k] = re;
                si[k] = im;
            }
            // lane 0 keeps A (k = 0) and sends its share of B; lane 1 keeps B
            const float keepR = h ? sr[1] : sr[0], keepI = h ? si[1] : si[0];
            const float sendR = h ? sr[0] : sr[1], sendI = h ? si[0] : si[1];
            float re = keepR + __shfl_xor_sync(0xffffffffu, sendR, 1);
            float im = keepI + __shfl_xor_sync(0xffffffffu, sendI, 1);
            const int p = pBase + u * 256;
            if (p < nOut) {
                if (p < K) {
                    if (cj[u]) im = -im;
                    store(row0 + i, p, re, im);
                    acc = fmaf(w2[u], re * re + im * im, acc);
                } else {
                    store(row0 + i, p, 0.f, 0.f);
                }
            }
        }
        if (nrmPart) {
            acc = warp_sum(acc);
            if (lane == 0) red[i][wid] = acc;
        }
    }
    if (nrmPart) {
        __syncthreads();
        if (threadIdx.x < nRot) {
            float s = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[threadIdx.x][w];
            nrmPart[(row0 + threadIdx.x) * nChunks + chunk] = s;
        }
    }
}

// FP32 rotation matrix of each projected row, from its quaternion
// (quat_to_mat in FP64, then rounded) or from an FP64 matrix.
__global__ void k_rot_f32(const double* __restrict__ quat, const double* __restrict__ mat,
                          int rows, float* __restrict__ mf)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        double md[9];
        if (quat) {
            double q[4] = {quat[4 * (size_t)r], quat[4 * (size_t)r + 1], quat[4 * (size_t)r + 2],
                           quat[4 * (size_t)r + 3]};
            quat_to_mat(q, md);
        } else {
            for (int i = 0; i < 9; i++) md[i] = mat[9 * (size_t)r + i];
        }
        for (int i = 0; i < 9; i++) mf[9 * (size_t)r + i] = (float)md[i];
    }
}

// nrm[row] = sum over the row's pixel chunks of nrmPart, in chunk order.
__global__ void k_norm_reduce(const float* __restrict__ nrmPart, int rows, int nChunks,
                              float* __restrict__ nrm)
{
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int c = 0; c < nChunks; c++) s += (double)nrmPart[(size_t)r * nChunks + c];
        nrm[r] = (float)s;
    }
}

// Shifted, weighted data A''[l][d][t][p] = sigRcp ctf_d X exp(+2 pi i (iCol tx
// + iRow ty) / N), the conjugate of sigRcp ctf_d conj(X) S_t, so that
// Re sum_p sigRcp ctf_d conj(X) S_t P = sum over the 2K floats of A'' . P.
// nD CTFs per particle (ctf [nP][nD][K]; one without a defocus search).
// CTA: (particle l, CTF d) x SHIFT_T translations; a thread loads its
// pixels' data, sigRcp and CTF once and writes them for every translation.
constexpr int SHIFT_T = 8;

__global__ void k_shift_bank(const float2* __restrict__ dat, const float* __restrict__ ctf,
                             const float* __restrict__ sigRcp,
                             const double* __restrict__ trans, const float2* __restrict__ bank,
                             int nT, int nD, int idim,
                             const int* __restrict__ iCol, const int* __restrict__ iRow,
                             int K, float* __restrict__ out, int ldo, long long splitLo,
                             int useTab, int tPer)
{
    // per-particle translations with useTab: the phase e^{2 pi i (iCol tx + iRow ty) / N}
    // is the product of a column factor and a row factor, tabulated once per
    // CTA for its translations (tabX [SHIFT_T][h + 1] over iCol = 0 .. h, tabY
    // [SHIFT_T][2h + 1] over iRow = -h .. h), so a pixel costs two shared
    // loads and a complex product instead of a sine and a cosine
    extern __shared__ float2 tabX[];
    const int ld = blockIdx.x;            // l nD + d
    const int l = ld / nD;
    // tPer (<= SHIFT_T) translations per CTA, spread evenly over the groups
    const int t0 = blockIdx.y * tPer;
    const int t1 = min(nT, t0 + tPer);
    const float invN = 1.0f / (float)idim;
    const int h = idim / 2, nc = h + 1, nr = 2 * h + 1;
    float2* tabY = tabX + SHIFT_T * nc;
    if (useTab && !bank) {
        for (int e = threadIdx.x; e < (t1 - t0) * (nc + nr); e += blockDim.x) {
            const int tt = e / (nc + nr), j = e % (nc + nr);
            const size_t lt = (size_t)l * nT + t0 + tt;
            float sn, cs;
            if (j < nc) {
                sincospif(2.0f * ((float)j * (float)trans[2 * lt]) * invN, &sn, &cs);
                tabX[tt * nc + j] = make_float2(cs, sn);
            } else {
                const int r = j - nc - h;
                sincospif(2.0f * ((float)r * (float)trans[2 * lt + 1]) * invN, &sn, &cs);
                tabY[tt * nr + (j - nc)] = make_float2(cs, sn);
            }
        }
        __syncthreads();
    }
    for (int p = threadIdx.x; p < ldo / 2; p += blockDim.x) {
        float sc = 0.f;
        float2 X = make_float2(0.f, 0.f);
        float fc = 0.f, fr = 0.f;
        int ic = 0, ir = 0;
        bool tabOk = false;
        if (p < K) {
            const size_t i = (size_t)l * K + p;
            sc = sigRcp[i] * ctf[(size_t)ld * K + p];
            X = dat[i];
            if (!bank) {
                ic = iCol[p];
                ir = iRow[p];
                fc = (float)ic;
                fr = (float)ir;
                tabOk = useTab && ic >= 0 && ic <= h && ir >= -h && ir <= h;
            }
        }
        for (int t = t0; t < t1; t++) {
            const size_t row = (size_t)ld * nT + t;     // (l nD + d) nT + t
            float2 v = make_float2(0.f, 0.f);
            if (p < K) {
                float s, c;
                if (bank) {
                    // shared phase bank S[t][p] = (cos, -sin): use conj(S)
                    const float2 S = bank[(size_t)t * K + p];
                    c = S.x;
                    s = -S.y;
                } else if (tabOk) {
                    const float2 ex = tabX[(t - t0) * nc + ic], ey = tabY[(t - t0) * nr + ir + h];
                    c = ex.x * ey.x - ex.y * ey.y;
                    s = ex.y * ey.x + ex.x * ey.y;
                } else {
                    const size_t lt = (size_t)l * nT + t;
                    const float tx = (float)trans[2 * lt], ty = (float)trans[2 * lt + 1];
                    float f = (fc * tx + fr * ty) * invN;
                    sincospif(2.0f * f, &s, &c);
                }
                v = make_float2(sc * (X.x * c - X.y * s), sc * (X.x * s + X.y * c));
            }
            store_pair(out, splitLo, row, ldo, p, v.x, v.y);
        }
    }
}

// Defocus search: the norm sum_p sigRcp ctf_d^2 |P|^2 of every projected row
// for each of the particle's nD CTFs, nrm[r][l][d] (the layout the weights
// kernel reads per (row, block)).  CTA: (particle, 8 rows), a warp per row,
// |P|^2 from the FP32 row or from the split planes (hi + lo).
constexpr int kMaxDefocus = 16;

__global__ void __launch_bounds__(256)
k_norm_defocus(const float* __restrict__ P, long long splitLo, int nP, int nR, int nD, int K,
               int Kp, const float* __restrict__ sigRcp, const float* __restrict__ ctf,
               float* __restrict__ nrm)
{
    const int l = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.y * 8 + warp;
    if (r >= nR) return;
    const size_t row = (size_t)l * nR + r;
    float acc[kMaxDefocus];
#pragma unroll
    for (int d = 0; d < kMaxDefocus; d++) acc[d] = 0.f;
    const __nv_bfloat162* hi = reinterpret_cast<const __nv_bfloat162*>(P);
    for (int p = lane; p < K; p += 32) {
        float re, im;
        if (splitLo == 0) {
            const float2 v = reinterpret_cast<const float2*>(P + row * Kp)[p];
            re = v.x;
            im = v.y;
        } else {
            const float2 h = __bfloat1622float2(hi[(row * Kp) / 2 + p]);
            const float2 o = __bfloat1622float2(hi[(splitLo + row * Kp) / 2 + p]);
            re = h.x + o.x;
            im = h.y + o.y;
        }
        const float a2 = sigRcp[(size_t)l * K + p] * (re * re + im * im);
#pragma unroll
        for (int d = 0; d < kMaxDefocus; d++) {
            if (d < nD) {
                const float c = ctf[((size_t)l * nD + d) * K + p];
                acc[d] = fmaf(a2, c * c, acc[d]);
            }
        }
    }
#pragma unroll
    for (int d = 0; d < kMaxDefocus; d++) {
        if (d >= nD) break;
        float v = acc[d];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) nrm[((size_t)r * nP + l) * nD + d] = v;
    }
}

// CTF of one particle for each defocus factor d (kernel_CalCTFL of the
// reference GPU path; the CTF of Optimiser::updateSP, src/Optimiser.cpp:
// 1196-1214): ki = k1 defO[p] d f[p]^2 + k2 f[p]^4 - phaseShift,
// ctf = -sqrt(1 - conT^2) sin ki + conT cos ki, in FP64; ctf [nD][K].
__global__ void k_ctf_defocus(const float* __restrict__ defO, const float* __restrict__ freQ,
                              const double* __restrict__ dpara, int K, double k1, double k2,
                              double phaseShift, double conT, float* __restrict__ ctf)
{
    const int d = blockIdx.y;
    const double w1 = sqrt(1.0 - conT * conT);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K; p += gridDim.x * blockDim.x) {
        const double f2 = (double)freQ[p] * freQ[p];
        const double ki = k1 * defO[p] * dpara[d] * f2 + k2 * f2 * f2 - phaseShift;
        ctf[(size_t)d * K + p] = (float)(-w1 * sin(ki) + conT * cos(ki));
    }
}

// 2-D projection (2-D classification): the bilinear sample of a class's
// half transform img [vdim][vdim/2 + 1] at the in-plane rotation (c, s) of
// every pixel (iCol pf, iRow pf): x = i c - j s, y = i s + j c (the
// reference's kernel_Project2D, gpu/src/Kernel.cu:786-819, reading as
// Image::getByInterpolationFT, src/Image/Image.cpp:345-368: x < 0 at (-x, -y)
// conjugated, rows wrapped).  Rows out [nR][ldo] as k_project writes them
// (FP32 pairs, or split planes when splitLo != 0), zero beyond K.
__global__ void k_project2d(const float2* __restrict__ img, int vdim, int pf,
                            const double* __restrict__ rot, const int* __restrict__ iCol,
                            const int* __restrict__ iRow, int K, float* __restrict__ out,
                            int ldo, long long splitLo)
{
    const int r = blockIdx.y;
    const float c = (float)rot[2 * (size_t)r], s = (float)rot[2 * (size_t)r + 1];
    const int nx = vdim / 2 + 1;
    const float fpf = (float)pf;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldo / 2;
         p += gridDim.x * blockDim.x) {
        float re = 0.f, im = 0.f;
        if (p < K) {
            const float i = (float)iCol[p] * fpf, j = (float)iRow[p] * fpf;
            float x = i * c - j * s, y = i * s + j * c;
            const bool conj = x < 0.f;
            if (conj) {
                x = -x;
                y = -y;
            }
            const float xf = floorf(x), yf = floorf(y);
            const int x0 = (int)xf, y0 = (int)yf;
            const float fx = x - xf, fy = y - yf;
#pragma unroll
            for (int b = 0; b < 2; b++) {
                int yy = y0 + b;
                yy = yy < 0 ? yy + vdim : yy;
                const float wy = b ? fy : 1.f - fy;
                const float2 v0 = __ldg(img + (size_t)yy * nx + x0);
                const float2 v1 = __ldg(img + (size_t)yy * nx + x0 + 1);
                re += wy * ((1.f - fx) * v0.x + fx * v1.x);
                im += wy * ((1.f - fx) * v0.y + fx * v1.y);
            }
            if (conj) im = -im;
        }
        store_pair(out, splitLo, r, ldo, p, re, im);
    }
}

// 2-D insertion (2-D classification; Reconstructor::insertP's 2-D form,
// Image::addFT(value, iCol, iRow), src/Image/Image.cpp:370-386; the
// reference's kernel_InsertF2D / T2D / O2D, gpu/src/Kernel.cu:2276-2470):
// draw d (image d / drawsPerImage, class nC[d], in-plane rotation nR[d] =
// (c, s), shift nT[d]) adds w ctf X shifted by -(t - offS) and w ctf^2
// bilinearly at (c a - s b, s a + c b), (a, b) = (iCol pf, iRow pf), into its
// class's (F.re, F.im, T, 0) accumulator [vdim][vdim/2 + 1] (x < 0: at
// (-x, -y), conjugated); O2D[class] gets -R (t - offS), counter[class] + 1.
// CTA (share of the pixels, draw).
__global__ void __launch_bounds__(256)
k_insert2d(float4* __restrict__ acc, int vdim, const float2* __restrict__ dat,
           const float* __restrict__ ctf, int ctfPerDraw, const float* __restrict__ wgt,
           const double* __restrict__ offS, const int* __restrict__ nC,
           const double* __restrict__ nR, const double* __restrict__ nT,
           const int* __restrict__ iCol, const int* __restrict__ iRow, int K, int pf, int idim,
           int d0, int drawsPerImage, double* __restrict__ O2D, int* __restrict__ counter)
{
    const int d = d0 + blockIdx.y;
    const int l = d / drawsPerImage;
    const int k = nC[d];
    const double cd = nR[2 * (size_t)d], sd = nR[2 * (size_t)d + 1];
    const double dx = nT[2 * (size_t)d] - offS[2 * (size_t)l];
    const double dy = nT[2 * (size_t)d + 1] - offS[2 * (size_t)l + 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (O2D) {
            atomicAdd(O2D + 2 * k, -(cd * dx - sd * dy));
            atomicAdd(O2D + 2 * k + 1, -(sd * dx + cd * dy));
        }
        if (counter) atomicAdd(counter + k, 1);
    }
    const int nx = vdim / 2 + 1;
    float4* a4 = acc + (size_t)k * vdim * nx;
    const float c = (float)cd, s = (float)sd, tx = (float)dx, ty = (float)dy, w = wgt[l];
    const float invN = 1.0f / (float)idim, fpf = (float)pf;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K; p += gridDim.x * blockDim.x) {
        const float2 X = dat[(size_t)l * K + p];
        const float cv = ctf[(ctfPerDraw ? (size_t)d : (size_t)l) * K + p];
        float sn, co;
        sincospif(2.0f * (((float)iCol[p] * tx + (float)iRow[p] * ty) * invN), &sn, &co);
        const float cw = cv * w;
        float vr = (X.x * co - X.y * sn) * cw, vi = (X.x * sn + X.y * co) * cw;
        const float vt = cv * cv * w;
        const float a = (float)iCol[p] * fpf, b = (float)iRow[p] * fpf;
        float x = c * a - s * b, y = s * a + c * b;
        if (x < 0.f) {
            x = -x;
            y = -y;
            vi = -vi;
        }
        const float xf = floorf(x), yf = floorf(y);
        const int x0 = (int)xf, y0 = (int)yf;
        const float fx = x - xf, fy = y - yf;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            int yy = y0 + j;
            yy = yy < 0 ? yy + vdim : yy;
            const float wy = j ? fy : 1.f - fy;
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const float ww = (i ? fx : 1.f - fx) * wy;
                atomicAdd(a4 + (size_t)yy * nx + x0 + i, make_float4(vr * ww, vi * ww, vt * ww, 0.f));
            }
        }
    }
}

// CTF attributes of every insertion draw with the defocus search: the
// image's attributes with defocusU, V scaled by the draw's factor nD (the
// defocus kernel_CalculateCTF uses, gpu/src/Kernel.cu:2132-2198).
__global__ void k_draw_attr(const float* __restrict__ attr, const double* __restrict__ nD,
                            int nDraws, int drawsPerImage, float* __restrict__ out)
{
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= nDraws) return;
    const float* a = attr + 7 * (size_t)(d / drawsPerImage);
    float* o = out + 7 * (size_t)d;
    for (int k = 0; k < 7; k++) o[k] = a[k];
    o[1] = (float)((double)a[1] * nD[d]);
    o[2] = (float)((double)a[2] * nD[d]);
}

// dst[(row nRep + k) len + j] = src[row len + j] (per-block copies of a
// particle's priors for the weights kernel's (particle, defocus) blocks)
__global__ void k_repeat_rows(const double* __restrict__ src, int rows, int len, int nRep,
                              double* __restrict__ dst)
{
    const size_t n = (size_t)rows * nRep * len;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t j = i % len, rk = i / len;
        dst[i] = src ? src[(rk / nRep) * len + j] : 1.0;
    }
}

// Merge of a particle's nD (particle, defocus) blocks, each relative to its
// own maximum, into the particle's weights relative to the overall maximum
// (the running baseline of Optimiser::updateSP, src/Optimiser.cpp:1326-1347,
// with its defocus axis): wD[d] = e_d wC_d, wC = sum_d pD[d] e_d wC_d,
// wR / wT = sum_d pD[d] e_d wR_d / wT_d, e_d = exp(base_d - base).
__global__ void k_merge_defocus(int nD, int nR, int nT, const double* __restrict__ wCb,
                                const double* __restrict__ wRb, const double* __restrict__ wTb,
                                const double* __restrict__ baseb, const double* __restrict__ pwD,
                                double* __restrict__ wC, double* __restrict__ wR,
                                double* __restrict__ wT, double* __restrict__ wD,
                                double* __restrict__ base)
{
    __shared__ double e[kMaxDefocus], pd[kMaxDefocus];
    const int l = blockIdx.x;
    if (threadIdx.x == 0) {
        double m = baseb[(size_t)l * nD];
        for (int d = 1; d < nD; d++) m = fmax(m, baseb[(size_t)l * nD + d]);
        double c = 0.0;
        for (int d = 0; d < nD; d++) {
            e[d] = exp(baseb[(size_t)l * nD + d] - m);
            pd[d] = pwD[(size_t)l * nD + d];
            wD[(size_t)l * nD + d] = e[d] * wCb[(size_t)l * nD + d];
            c += pd[d] * wD[(size_t)l * nD + d];
        }
        wC[l] = c;
        base[l] = m;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < nR; r += blockDim.x) {
        double s = 0.0;
        for (int d = 0; d < nD; d++) s += pd[d] * e[d] * wRb[((size_t)l * nD + d) * nR + r];
        wR[(size_t)l * nR + r] = s;
    }
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        double s = 0.0;
        for (int d = 0; d < nD; d++) s += pd[d] * e[d] * wTb[((size_t)l * nD + d) * nT + t];
        wT[(size_t)l * nT + t] = s;
    }
}

__global__ void k_x0(const float2* __restrict__ dat, const float* __restrict__ sigRcp,
                     int K, double* __restrict__ x0)
{
    __shared__ double red[32];
    const int l = blockIdx.x;
    double acc = 0;
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        // FP32 terms, FP64 sum: one double add a pixel (the GPU's FP64
        // rate is a small fraction of its FP32 rate)
        const float2 X = dat[(size_t)l * K + p];
        acc += (double)(sigRcp[(size_t)l * K + p] * fmaf(X.x, X.x, X.y * X.y));
    }
    double s = block_sum_d(acc, red);
    if (threadIdx.x == 0) x0[l] = s;
}

// ------------------------------------------------------------------------
// Batched FP32 "NT" GEMM on the CUDA cores: C[b][i][j] = alpha sum_k
// A[b][i][k] B[b][j][k] (+ nrm[b][i]).  128 x 128 x 16 tiles, 256 threads,
// 8 x 8 outputs per thread, register-staged double buffering.  Kd must be a
// multiple of 16 and lda/ldb multiples of 4 (rows zero-padded).
constexpr int GB_M = 128, GB_N = 128, GB_K = 16, GB_PAD = 4;

__global__ void __launch_bounds__(256, 1)
k_gemm_nt_fp32(const float* __restrict__ A, long long sA, int lda,
               const float* __restrict__ B, long long sB, int ldb,
               int M, int N, int Kd, float* __restrict__ C, long long sC, int ldc,
               const float* __restrict__ nrm, long long sN, float alpha, int cGroup,
               long long cGroupStride)
{
    __shared__ __align__(16) float As[2][GB_K][GB_M + GB_PAD];
    __shared__ __align__(16) float Bs[2][GB_K][GB_N + GB_PAD];
    const int b = blockIdx.z;
    const int i0 = blockIdx.y * GB_M, j0 = blockIdx.x * GB_N;
    A += b * sA;
    B += b * sB;
    C += b * sC;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    // loader mapping: two float4 per operand per k-tile (rows lr and lr + 64)
    const int lr = tid >> 2, lk = (tid & 3) * 4;
    const bool a0ok = i0 + lr < M, a1ok = i0 + lr + 64 < M;
    const bool b0ok = j0 + lr < N, b1ok = j0 + lr + 64 < N;
    const float* Ap0 = A + (size_t)(a0ok ? i0 + lr : 0) * lda + lk;
    const float* Ap1 = A + (size_t)(a1ok ? i0 + lr + 64 : 0) * lda + lk;
    const float* Bp0 = B + (size_t)(b0ok ? j0 + lr : 0) * ldb + lk;
    const float* Bp1 = B + (size_t)(b1ok ? j0 + lr + 64 : 0) * ldb + lk;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.f;

    float4 ra[2], rb[2];
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    ra[0] = a0ok ? __ldg(reinterpret_cast<const float4*>(Ap0)) : z4;
    ra[1] = a1ok ? __ldg(reinterpret_cast<const float4*>(Ap1)) : z4;
    rb[0] = b0ok ? __ldg(reinterpret_cast<const float4*>(Bp0)) : z4;
    rb[1] = b1ok ? __ldg(reinterpret_cast<const float4*>(Bp1)) : z4;
    const int nk = Kd / GB_K;
    int buf = 0;
    for (int kt = 0; kt < nk; kt++) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            As[buf][lk + 0][lr + 64 * h] = ra[h].x;
            As[buf][lk + 1][lr + 64 * h] = ra[h].y;
            As[buf][lk + 2][lr + 64 * h] = ra[h].z;
            As[buf][lk + 3][lr + 64 * h] = ra[h].w;
            Bs[buf][lk + 0][lr + 64 * h] = rb[h].x;
            Bs[buf][lk + 1][lr + 64 * h] = rb[h].y;
            Bs[buf][lk + 2][lr + 64 * h] = rb[h].z;
            Bs[buf][lk + 3][lr + 64 * h] = rb[h].w;
        }
        __syncthreads();
        if (kt + 1 < nk) {
            const int off = (kt + 1) * GB_K;
            ra[0] = a0ok ? __ldg(reinterpret_cast<const float4*>(Ap0 + off)) : z4;
            ra[1] = a1ok ? __ldg(reinterpret_cast<const float4*>(Ap1 + off)) : z4;
            rb[0] = b0ok ? __ldg(reinterpret_cast<const float4*>(Bp0 + off)) : z4;
            rb[1] = b1ok ? __ldg(reinterpret_cast<const float4*>(Bp1 + off)) : z4;
        }
#pragma unroll
        for (int kk = 0; kk < GB_K; kk++) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
            const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        buf ^= 1;
    }
    // epilogue
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int gi = i0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (gi >= M) continue;
        const float add = nrm ? nrm[b * sN + gi] : 0.f;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int gj = j0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + (j - 4));
            if (gj < N) {
                size_t off = (size_t)gi * ldc + gj;
                if (cGroup > 0) {
                    const int l = gj / cGroup;
                    off = (size_t)l * cGroupStride + (size_t)gi * ldc + (gj - l * cGroup);
                }
                C[off] = fmaf(alpha, acc[i][j], add);
            }
        }
    }
}

// ------------------------------------------------------------------------
// Marginal weights of one hypothesis block (a particle, or an image of the
// global scan): base = max D, s = exp(D - base),
//   wR[r] = sum_t s pwC pwT[t], wT[t] = sum_r s pwC pwR[r],
//   wC = sum s pwR[r] pwT[t]
// (the running-baseline accumulation of Optimiser::updateSP,
// src/Optimiser.cpp:1326-1347, evaluated in two passes).  D of block (b, g)
// is D[b sD + r ldc + g nT + t].  One CTA of 512 threads per block; a warp
// takes whole rotation rows (lanes over translations, coalesced), sums wR[r]
// with shuffles, and keeps its share of wT in registers (TS slots of 32
// translations; TS == 0: shared-memory atomics for long rows).  FP32
// accumulation, as in the reference GPU path; totals are combined in FP64.
// Callers with many small blocks (the multi-class scan) may launch fewer
// warps, so that the per-warp fixed work -- reductions, loop set-up -- is
// spread over more rows; the warp count sets the order of the wT sums.
constexpr int WEIGHTS_THREADS = 512;

template <int TS>
__global__ void __launch_bounds__(WEIGHTS_THREADS)
k_weights(const float* __restrict__ D, long long sD, int ldc, int nR, int nT, int G,
          const float* __restrict__ nrmG, int nrmRS, const double* __restrict__ x0,
          const double* __restrict__ pwR, long long sR,
          const double* __restrict__ pwT, long long sT, const double* __restrict__ pwC,
          double* __restrict__ wC, double* __restrict__ wR, double* __restrict__ wT,
          double* __restrict__ base, float* __restrict__ dvp, int nc)
{
    extern __shared__ float wsm[];
    float* wTs = wsm;                // [nT]
    float* pTs = wTs + nT;           // [nT]
    float* wTw = pTs + nT;           // [warps][nT] when TS > 0: per-warp sums, added in order
    __shared__ float redf[32];
    __shared__ double red[32];
    // nc > 1: the rows of item blk / nc are cut into nc chunks, one per CTA;
    // wC, wT, base are then per chunk (relative to the chunk's maximum) and
    // k_merge_chunks folds them; wR and dvp rows go straight to the item's
    const int blk = blockIdx.x;
    const int item = blk / nc, chunk = blk % nc;
    const int rpb = (nR + nc - 1) / nc;
    const int r0c = min(nR, chunk * rpb);
    const int nRc = min(nR, r0c + rpb) - r0c;
    const int b = item / G, g = item % G;
    const float* Db = D + b * sD + (size_t)g * nT + (size_t)r0c * ldc;
    const double* pr = pwR + item * sR + r0c;
    const double* pt = pwT + item * sT;
    const double pc = pwC ? pwC[item] : 1.0;
    const float* nrmB = nrmG ? nrmG + (size_t)r0c * nrmRS : nullptr;
    const int nRall = nR;
    nR = nRc;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        wTs[t] = 0.f;
        pTs[t] = (float)pt[t];
    }
    // pass 1: maximum (four rows per warp in flight)
    float mx = -CUDART_INF_F;
    for (int r0 = wid; r0 < nR; r0 += 4 * nw) {
        float v[4][TS > 0 ? TS : 1];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int r = r0 + q * nw;
            const float ad = (r < nR && nrmB) ? nrmB[(size_t)r * nrmRS + item] : 0.f;
            const float* row = Db + (size_t)(r < nR ? r : 0) * ldc;
#pragma unroll
            for (int j = 0; j < (TS > 0 ? TS : 1); j++) {
                const int t = lane + 32 * j;
                v[q][j] = (r < nR && t < nT && TS > 0) ? row[t] + ad : -CUDART_INF_F;
            }
            if (TS == 0 && r < nR)
                for (int t = lane; t < nT; t += 32) mx = fmaxf(mx, row[t] + ad);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
#pragma unroll
            for (int j = 0; j < (TS > 0 ? TS : 1); j++) mx = fmaxf(mx, v[q][j]);
    }
    mx = warp_max(mx);
    if (lane == 0) redf[wid] = mx;
    __syncthreads();
    if (wid == 0) {
        float v = lane < nw ? redf[lane] : -CUDART_INF_F;
        v = warp_max(v);
        if (lane == 0) redf[0] = v;
    }
    __syncthreads();
    const float M = redf[0];
    const double x0b = x0 ? x0[item] : 0.0;
    // pass 2: marginals
    float tacc[TS > 0 ? TS : 1], ptv[TS > 0 ? TS : 1];
#pragma unroll
    for (int j = 0; j < (TS > 0 ? TS : 1); j++) {
        tacc[j] = 0.f;
        const int t = lane + 32 * j;
        ptv[j] = (TS > 0 && t < nT) ? pTs[t] : 0.f;
    }
    float cacc = 0.f;
    // two rows per warp in flight: both rows' loads precede their arithmetic
    for (int r0 = wid; r0 < nR; r0 += 2 * nw) {
        float dv[2][TS > 0 ? TS : 1], prr[2], ad[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int r = r0 + q * nw;
            const bool rok = r < nR;
            prr[q] = rok ? (float)pr[r] : 0.f;
            ad[q] = (rok && nrmB) ? nrmB[(size_t)r * nrmRS + item] : 0.f;
            const float* row = Db + (size_t)(rok ? r : 0) * ldc;
#pragma unroll
            for (int j = 0; j < (TS > 0 ? TS : 1); j++) {
                const int t = lane + 32 * j;
                dv[q][j] = (TS > 0 && rok && t < nT) ? row[t] : 0.f;
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const int r = r0 + q * nw;
            if (r >= nR) break;
            const float* row = Db + (size_t)r * ldc;
            float racc = 0.f;
            if (TS > 0) {
#pragma unroll
                for (int j = 0; j < (TS > 0 ? TS : 1); j++) {
                    const int t = lane + 32 * j;
                    if (t < nT) {
                        const float d = dv[q][j] + ad[q];
                        const float sv = __expf(d - M);
                        racc = fmaf(sv, ptv[j], racc);
                        tacc[j] = fmaf(sv, prr[q], tacc[j]);
                        if (dvp)
                            dvp[((size_t)item * nRall + r0c + r) * nT + t] =
                                (float)(x0b + (double)d);
                    }
                }
            } else {
                for (int t = lane; t < nT; t += 32) {
                    const float d = row[t] + ad[q];
                    const float sv = __expf(d - M);
                    racc = fmaf(sv, pTs[t], racc);
                    atomicAdd(wTs + t, sv * prr[q]);
                    if (dvp)
                        dvp[((size_t)item * nRall + r0c + r) * nT + t] =
                            (float)(x0b + (double)d);
                }
            }
            racc = warp_sum(racc);
            cacc = fmaf(racc, prr[q], cacc);   // sum_t s pT[t] pR[r], once per row
            if (lane == 0) wR[(size_t)item * nRall + r0c + r] = (double)racc * pc;
        }
    }
    if (TS > 0) {
#pragma unroll
        for (int j = 0; j < (TS > 0 ? TS : 1); j++) {
            const int t = lane + 32 * j;
            if (t < nT) wTw[wid * nT + t] = tacc[j];
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        float v = wTs[t];
        if (TS > 0) {
            // the warps' sums in warp order: the same bits on every run
            v = 0.f;
            for (int w = 0; w < nw; w++) v += wTw[w * nT + t];
        }
        wT[(size_t)blk * nT + t] = (double)v * pc;
    }
    // every lane holds the same cacc per warp: count lane 0's only
    const double c = block_sum_d(lane == 0 ? (double)cacc : 0.0, red);
    if (threadIdx.x == 0) {
        wC[blk] = c;
        base[blk] = x0b + (double)M;
    }
}

// Fold the weights of class kIdx into the reference's running per-image
// layout: wC [img][nK], wR [img][nK][nR], wT [img][nK][nT] relative to baseL
// (kernel_setBaseLine / kernel_UpdateW of the reference GPU path, with the
// CPU scan's rescale rule, src/Optimiser.cpp:835-898).
// The class's inputs of image l are wCn[l s], wRn[l s nR + r], wTn[l s nT + t],
// basen[l s], s = inStride (1: one class's arrays; nK: a class's column of
// per-(image, class) arrays).
__global__ void k_merge_class(int nK, int kIdx, int nR, int nT,
                              const double* __restrict__ wCn, const double* __restrict__ wRn,
                              const double* __restrict__ wTn, const double* __restrict__ basen,
                              float* __restrict__ wC, float* __restrict__ wR,
                              float* __restrict__ wT, float* __restrict__ baseL, int inStride)
{
    const int l = blockIdx.x;
    const size_t li = (size_t)l * inStride;
    const double bn = basen[li];
    double scaleOld = 0.0, scaleNew = 1.0, newBase = bn;
    if (kIdx > 0) {
        const double bo = baseL[l];
        if (bn > bo) { scaleOld = exp(bo - bn); newBase = bn; }
        else { scaleOld = 1.0; scaleNew = exp(bn - bo); newBase = bo; }
    }
    __syncthreads();
    for (int k = 0; k < nK; k++) {
        const bool cur = (k == kIdx);
        if (!cur && (kIdx == 0 || k > kIdx)) {
            // classes not yet scored: zero on the first class only
            if (kIdx == 0) {
                if (threadIdx.x == 0) wC[(size_t)l * nK + k] = 0.f;
                for (int r = threadIdx.x; r < nR; r += blockDim.x) wR[((size_t)l * nK + k) * nR + r] = 0.f;
                for (int t = threadIdx.x; t < nT; t += blockDim.x) wT[((size_t)l * nK + k) * nT + t] = 0.f;
            }
            continue;
        }
        if (cur) {
            if (threadIdx.x == 0) wC[(size_t)l * nK + k] = (float)(wCn[li] * scaleNew);
            for (int r = threadIdx.x; r < nR; r += blockDim.x)
                wR[((size_t)l * nK + k) * nR + r] = (float)(wRn[li * nR + r] * scaleNew);
            for (int t = threadIdx.x; t < nT; t += blockDim.x)
                wT[((size_t)l * nK + k) * nT + t] = (float)(wTn[li * nT + t] * scaleNew);
        } else if (scaleOld != 1.0) {
            if (threadIdx.x == 0) wC[(size_t)l * nK + k] = (float)(wC[(size_t)l * nK + k] * scaleOld);
            for (int r = threadIdx.x; r < nR; r += blockDim.x)
                wR[((size_t)l * nK + k) * nR + r] = (float)(wR[((size_t)l * nK + k) * nR + r] * scaleOld);
            for (int t = threadIdx.x; t < nT; t += blockDim.x)
                wT[((size_t)l * nK + k) * nT + t] = (float)(wT[((size_t)l * nK + k) * nT + t] * scaleOld);
        }
    }
    if (threadIdx.x == 0) baseL[l] = (float)newBase;
}

// ------------------------------------------------------------------------
// Narrowing + systematic resampling of one axis of one particle per CTA
// (Particle::keepHalfHeightPeak, src/Particle.cpp:1935-1973;
//  Particle::shuffle, :2173-2270; Particle::resample(n, pt), :1275-1463;
//  Particle::normW, :813-820; Particle::setPeakFactor(PAR_R) 3D, :1886-1896).
// Sums and the cumulative sum run sequentially in one thread so that every
// result is bit-identical to the reference's sequential double arithmetic;
// the draws use a binary search, which finds the same first index with
// cdf >= u_j as the reference's forward scan.
__global__ void __launch_bounds__(256)
k_resample(int ld, const double* __restrict__ uIn, const double* __restrict__ wIn,
           const int* __restrict__ perm, const double* __restrict__ u0s,
           const double* __restrict__ peaks, int ldo, const int* __restrict__ nPer,
           int* __restrict__ src, double* __restrict__ wOut, int* __restrict__ top,
           int* __restrict__ flag)
{
    // ld / ldo: pitches of the inputs / outputs of a particle; its own set has
    // n = nPer[b] entries (all ld without nPer) and it draws nOut = n of them
    // (ldo without nPer)
    extern __shared__ double sm[];
    double* u = sm;                 // [ld]
    double* w = u + ld;             // [ld]
    double* cdf = w + ld;           // [max(ld, ldo)]
    int* idx = reinterpret_cast<int*>(cdf + (ld > ldo ? ld : ldo));   // [ld]
    __shared__ double sval[32];
    __shared__ int sidx[32];
    __shared__ double sh;
    __shared__ int bad;
    const int b = blockIdx.x;
    const int n = nPer ? nPer[b] : ld;
    const int nOut = nPer ? n : ldo;
    const double* ub = uIn + (size_t)b * ld;
    const double* wb = wIn + (size_t)b * ld;
    const int* pb = perm + (size_t)b * ld;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) bad = 0;
    // maximum of u (exact in any order)
    double mx = -CUDART_INF;
    for (int i = threadIdx.x; i < n; i += blockDim.x) mx = fmax(mx, ub[i]);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) sval[wid] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = sval[0];
        for (int i = 1; i < nw; i++) m = fmax(m, sval[i]);
        sh = m;
    }
    __syncthreads();
    const double umax = sh;
    double pf = peaks ? peaks[b] : 0.0;
    if (isnan(pf)) {
        // value of rank n/8 in descending order (Particle::setPeakFactor)
        // The rank count compares monotone integer keys of the doubles (the
        // IEEE bit pattern, negatives reflected): exact, and integer compares
        // run at full rate where FP64 compares would not.
        const int k = n / 8;
        long long* key = reinterpret_cast<long long*>(cdf);   // cdf is unused yet
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double x = ub[i];
            const long long bits = __double_as_longlong(x == 0.0 ? 0.0 : x);
            key[i] = bits ^ ((bits >> 63) & 0x7fffffffffffffffLL);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const long long v = key[i];
            int gt = 0, ge = 0;
            for (int j = 0; j < n; j++) {
                const long long x = key[j];
                gt += x > v;
                ge += x >= v;
            }
            if (gt <= k && k < ge) sh = ub[i];   // all writers store the same value
        }
        __syncthreads();
        const double r = __ddiv_rn(sh, umax);
        pf = fmax(1e-3, fmin(0.5, r));
        __syncthreads();
    }
    const double hh = pf > 0 ? __dmul_rn(umax, pf) : 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double ui = ub[i];
        if (pf > 0) ui = (ui < hh) ? 0.0 : __dsub_rn(ui, hh);
        const int d = pb[i];
        if (d < 0 || d >= n) { bad = 1; continue; }
        u[d] = ui;
        w[d] = wb[i];
        idx[d] = i;
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) atomicOr(flag, 1);
        return;
    }
    // best sample, last index among equal maxima (gsl_sort_largest_index)
    double bv = -CUDART_INF;
    int bi = -1;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (u[i] >= bv) { bv = u[i]; bi = i; }
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_xor_sync(0xffffffffu, bv, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi > bi)) { bv = ov; bi = oi; }
    }
    if (lane == 0) { sval[wid] = bv; sidx[wid] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = sval[0];
        int ii = sidx[0];
        for (int i = 1; i < nw; i++)
            if (sval[i] > v || (sval[i] == v && sidx[i] > ii)) { v = sval[i]; ii = sidx[i]; }
        top[b] = ii >= 0 ? idx[ii] : 0;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = __dmul_rn(w[i], u[i]);
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = w[0];
        for (int i = 1; i < n; i++) s = __dadd_rn(s, w[i]);
        sh = s;
    }
    __syncthreads();
    const double ws = sh;
    if (!(ws > 0.0)) {
        if (threadIdx.x == 0) atomicOr(flag, 2);
        return;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] = __ddiv_rn(w[i], ws);
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int i = 0; i < n; i++) { acc = __dadd_rn(acc, w[i]); cdf[i] = acc; }
    }
    __syncthreads();
    const double last = cdf[n - 1];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) cdf[i] = __ddiv_rn(cdf[i], last);
    __syncthreads();
    const double u0 = u0s[b];
    int* so = src + (size_t)b * ldo;
    for (int j = threadIdx.x; j < nOut; j += blockDim.x) {
        const double uj = __dadd_rn(u0, __ddiv_rn((double)j, (double)nOut));
        int lo = 0, hi = n - 1;       // first i with cdf[i] >= uj
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (uj > cdf[mid]) lo = mid + 1; else hi = mid;
        }
        so[j] = idx[lo];
        // new prior 1 / u of the source (PARTICLE_PRIOR_ONE)
        wOut[(size_t)b * ldo + j] = __ddiv_rn(1.0, u[lo]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double* wb2 = wOut + (size_t)b * ldo;
        double s = wb2[0];
        for (int j = 1; j < nOut; j++) s = __dadd_rn(s, wb2[j]);
        sh = s;
    }
    __syncthreads();
    const double s2 = sh;
    for (int j = threadIdx.x; j < nOut; j += blockDim.x)
        wOut[(size_t)b * ldo + j] = __ddiv_rn(wOut[(size_t)b * ldo + j], s2);
}

// ------------------------------------------------------------------------
// Insertion of one weighted, shifted slice per CTA into the interleaved
// (F.re, F.im, T, 0) accumulator (Reconstructor::insertP,
// src/Reconstructor.cpp:782-863).  The image is first shifted by
// -(t - offset) (translate, src/Image/ImageFunctions.cpp:471-492, as in
// Optimiser::reconstructRef, src/Optimiser.cpp:7115-7136).
//   MKB: every voxel with tab[rint(r^2 n / b)] != 0 inside the radius
//        (Volume::addFT(value, x, y, z, a, TabFunction),
//        src/Image/Volume.cpp:399-431; entries past the kernel support are
//        zero, so the loop covers only the support);
//   trilinear: the eight corners (Volume::addFT(value, x, y, z),
//        src/Image/Volume.cpp:334-369).
// Voxels with x < 0 are mirrored and conjugated (Volume::iFT).
__device__ __forceinline__ void red_voxel(float4* acc, int vdim, int nx, int i, int j, int k,
                                          float fr, float fi, float t)
{
    if (i < 0) { i = -i; j = -j; k = -k; fi = -fi; }
    const int yy = j < 0 ? j + vdim : j, zz = k < 0 ? k + vdim : k;
    float4* p = acc + ((size_t)zz * vdim + yy) * nx + i;
    atomicAdd(p, make_float4(fr, fi, t, 0.f));
}

// Per-draw parameters of the insertion, one thread per draw: the FP32
// rotation (quat_to_mat in FP64, rounded), the shift t - offset and the
// image weight, 16 floats per draw; and the bookkeeping: O3D -= R (t -
// offset, 0) (insertDir, src/Optimiser.cpp:7180-7186), summed per block
// before one atomic per component, and the draw counter.
// With nC (the multi-class InsertFT), draw m of image l is inserted only
// when m < nC[l] (kernel_getRandomR / kernel_InsertF, gpu/src/Kernel.cu:
// 1847-1899, 2552-2600): a skipped draw gets weight 0, which k_insert
// skips, and adds nothing to O3D or the counter.
__global__ void __launch_bounds__(256)
k_insert_draws(int nDraws, int drawsPerImage, const double* __restrict__ quat,
               const double* __restrict__ trans, const double* __restrict__ offset,
               const float* __restrict__ wgt, float* __restrict__ params,
               double* __restrict__ O3D, int* __restrict__ counter, const int* __restrict__ nC)
{
    __shared__ double part[3][8];
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    double o[3] = {0.0, 0.0, 0.0};
    const bool active = d < nDraws && (!nC || d % drawsPerImage < nC[d / drawsPerImage]);
    if (d < nDraws && !active) {
        float* pd = params + 16 * (size_t)d;
        for (int i = 0; i < 12; i++) pd[i] = 0.f;
    }
    if (active) {
        const int l = d / drawsPerImage;
        double q[4] = {quat[4 * (size_t)d], quat[4 * (size_t)d + 1], quat[4 * (size_t)d + 2],
                       quat[4 * (size_t)d + 3]};
        double md[9];
        quat_to_mat(q, md);
        const double tx = trans[2 * (size_t)d] - (offset ? offset[2 * (size_t)l] : 0.0);
        const double ty = trans[2 * (size_t)d + 1] - (offset ? offset[2 * (size_t)l + 1] : 0.0);
        float* pd = params + 16 * (size_t)d;
        for (int i = 0; i < 9; i++) pd[i] = (float)md[i];
        pd[9] = (float)tx;
        pd[10] = (float)ty;
        pd[11] = wgt[l];
        o[0] = -(md[0] * tx + md[1] * ty);
        o[1] = -(md[3] * tx + md[4] * ty);
        o[2] = -(md[6] * tx + md[7] * ty);
    }
    if (O3D) {
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int k = 0; k < 3; k++) {
            double v = o[k];
            for (int sft = 16; sft; sft >>= 1) v += __shfl_xor_sync(0xffffffffu, v, sft);
            if (lane == 0) part[k][wid] = v;
        }
        __syncthreads();
        if (threadIdx.x < 3) {
            double v = 0.0;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += part[threadIdx.x][w];
            atomicAdd(O3D + threadIdx.x, v);
        }
    }
    if (counter) {
        const int n = __syncthreads_count(active);
        if (threadIdx.x == 0 && n > 0) atomicAdd(counter, n);
    }
}

// CTA (share of the pixels, draw); parameters from k_insert_draws.
__global__ void __launch_bounds__(256)
k_insert(float4* __restrict__ acc, int vdim, int kernel, const float* __restrict__ tab,
         int tabNz, float tabInvStep, float rs2, const float2* __restrict__ dat,
         const float* __restrict__ ctf, const float* __restrict__ params,
         const int* __restrict__ iCol, const int* __restrict__ iRow, int K, int pf, int idim,
         int d0, int drawsPerImage, int ctfPerDraw)
{
    const int d = d0 + blockIdx.y;            // draw; blockIdx.x: share of its pixels
    const int l = d / drawsPerImage;          // image
    const float* pd = params + 16 * (size_t)d;
    float m[9];
#pragma unroll
    for (int i = 0; i < 9; i++) m[i] = __ldg(pd + i);
    const int nx = vdim / 2 + 1, half = vdim / 2;
    const float tx = __ldg(pd + 9), ty = __ldg(pd + 10), w = __ldg(pd + 11);
    if (w == 0.f) return;                     // a skipped draw (or one of weight 0)
    const float invN = 1.0f / (float)idim;
    const float fpf = (float)pf;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < K; p += gridDim.x * blockDim.x) {
        const size_t di = (size_t)l * K + p;
        const float c = ctf[(ctfPerDraw ? (size_t)d : (size_t)l) * K + p];
        const float2 X = dat[di];
        // shift by -(t - offset): multiply by exp(+2 pi i k.t / N)
        float f = ((float)iCol[p] * tx + (float)iRow[p] * ty) * invN;
        float s, co;
        sincospif(2.0f * f, &s, &co);
        const float cw = c * w;
        const float vr = (X.x * co - X.y * s) * cw, vi = (X.x * s + X.y * co) * cw;
        const float vt = c * c * w;
        const float a = (float)iCol[p] * fpf, b = (float)iRow[p] * fpf;
        float x = m[0] * a + m[1] * b;
        float y = m[3] * a + m[4] * b;
        float z = m[6] * a + m[7] * b;
        if (kernel == TG3_KERNEL_MKB) {
            // every voxel with rint(r^2 n / b) <= tabNz has r^2 < rs2: per
            // axis, only the lattice points inside that sphere are visited
            const float rs = sqrtf(rs2);
            const int k0 = max(-half, (int)ceilf(z - rs)), k1 = min(half - 1, (int)floorf(z + rs));
            for (int kk = k0; kk <= k1; kk++) {
                const float dz = z - (float)kk;
                const float sz = rs2 - dz * dz;
                if (sz < 0.f) continue;
                const float ry = sqrtf(sz);
                const int j0 = max(-half, (int)ceilf(y - ry));
                const int j1 = min(half - 1, (int)floorf(y + ry));
                for (int jj = j0; jj <= j1; jj++) {
                    const float dy = y - (float)jj;
                    const float dyz = dy * dy + dz * dz;
                    const float sx = rs2 - dyz;
                    if (sx < 0.f) continue;
                    const float rx = sqrtf(sx);
                    const int i0 = max(-half, (int)ceilf(x - rx));
                    const int i1 = min(half, (int)floorf(x + rx));
                    // at most 4 lattice points (2 rx < 4, checked by the
                    // launcher): the row's table loads are issued together
                    int tv[4];
                    float kv[4];
#pragma unroll
                    for (int v = 0; v < 4; v++) {
                        const float dx = x - (float)(i0 + v);
                        const int ti = __float2int_rn((dx * dx + dyz) * tabInvStep);
                        tv[v] = (i0 + v <= i1 && ti <= tabNz) ? ti : -1;
                        kv[v] = tv[v] >= 0 ? __ldg(tab + tv[v]) : 0.f;
                    }
#pragma unroll
                    for (int v = 0; v < 4; v++)
                        if (tv[v] >= 0)
                            red_voxel(acc, vdim, nx, i0 + v, jj, kk, vr * kv[v], vi * kv[v],
                                      vt * kv[v]);
                }
            }
        } else {
            float fi = vi;
            if (x < 0.f) { x = -x; y = -y; z = -z; fi = -fi; }
            const float xf = floorf(x), yf = floorf(y), zf = floorf(z);
            const int x0 = (int)xf, y0 = (int)yf, z0 = (int)zf;
            const float fx = x - xf, fy = y - yf, fz = z - zf;
            const float wx[2] = {1.f - fx, fx}, wy[2] = {1.f - fy, fy}, wz[2] = {1.f - fz, fz};
#pragma unroll
            for (int k = 0; k < 2; k++)
#pragma unroll
                for (int j = 0; j < 2; j++)
#pragma unroll
                    for (int i = 0; i < 2; i++) {
                        const float ww = wx[i] * wy[j] * wz[k];
                        int yy = y0 + j, zz = z0 + k;
                        yy = yy < 0 ? yy + vdim : yy;
                        zz = zz < 0 ? zz + vdim : zz;
                        atomicAdd(acc + ((size_t)zz * vdim + yy) * nx + (x0 + i),
                                  make_float4(vr * ww, fi * ww, vt * ww, 0.f));
                    }
        }
    }
}

// ------------------------------------------------------------------------
// MKB insertion as a gather (same sums as k_insert, one atomic per voxel).
//
// Stage: CTA (tile, draw) writes cells of the draw's dense half-plane grid
// [2 Rg + 1 rows][Rg + 1 columns] of float4: the shifted, weighted value
// (c w X e^{2 pi i k.t/N}, c^2 w) of the cell's pixel, zero where no pixel
// lies (cellPix < 0).  CTA (0, draw) also writes the draw's FP32 rotation
// and does its bookkeeping (O3D, counter) exactly as k_insert.
__global__ void __launch_bounds__(256)
k_insert_stage(float4* __restrict__ grid, int cells, float* __restrict__ rot,
               const int* __restrict__ cellPix, const int* __restrict__ iCol,
               const int* __restrict__ iRow, const float2* __restrict__ dat,
               const float* __restrict__ ctf, const double* __restrict__ quat,
               const double* __restrict__ trans, const double* __restrict__ offset,
               const float* __restrict__ wgt, int K, int idim, int d0, int drawsPerImage,
               int ctfPerDraw, double* __restrict__ O3D, int* __restrict__ counter)
{
    const int dl = blockIdx.y;                // draw within the chunk
    const int d = d0 + dl;
    const int l = d / drawsPerImage;
    const double txd = trans[2 * (size_t)d] - (offset ? offset[2 * (size_t)l] : 0.0);
    const double tyd = trans[2 * (size_t)d + 1] - (offset ? offset[2 * (size_t)l + 1] : 0.0);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        double q[4] = {quat[4 * (size_t)d], quat[4 * (size_t)d + 1], quat[4 * (size_t)d + 2],
                       quat[4 * (size_t)d + 3]};
        double md[9];
        quat_to_mat(q, md);
        for (int i = 0; i < 9; i++) rot[16 * (size_t)dl + i] = (float)md[i];
        if (O3D) {
            atomicAdd(O3D + 0, -(md[0] * txd + md[1] * tyd));
            atomicAdd(O3D + 1, -(md[3] * txd + md[4] * tyd));
            atomicAdd(O3D + 2, -(md[6] * txd + md[7] * tyd));
        }
        if (counter) atomicAdd(counter, 1);
    }
    const float tx = (float)txd, ty = (float)tyd, w = wgt[l];
    const float invN = 1.0f / (float)idim;
    float4* g = grid + (size_t)dl * cells;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cells; i += gridDim.x * blockDim.x) {
        const int p = cellPix[i];
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p >= 0) {
            const size_t di = (size_t)l * K + p;
            const float c = ctf[(ctfPerDraw ? (size_t)d : (size_t)l) * K + p];
            const float2 X = dat[di];
            float f = ((float)iCol[p] * tx + (float)iRow[p] * ty) * invN;
            float sn, co;
            sincospif(2.0f * f, &sn, &co);
            const float cw = c * w;
            v = make_float4((X.x * co - X.y * sn) * cw, (X.x * sn + X.y * co) * cw, c * c * w,
                            0.f);
        }
        g[i] = v;
    }
}

// Gather: CTA (tile, draw); each thread takes rows (x-runs of fixed y, z) of
// the stored half volume that cross the draw's slab |h| <= hs, h = e3 . v,
// inside the cylinder of in-plane radius Rp + hs.  Each voxel v = (x, y, z)
// takes its plane coordinates (a, b, h) = R^T v and sums the MKB-weighted
// values of the grid cells within the support: a pixel (c, r) at
// (pf c, pf r, 0) directly, and, for x > 0, the Friedel mate of pixel (c, r)
// at (-pf c, -pf r, 0), conjugated.  This is the set of writes k_insert
// makes to v (direct writes to x >= 0, mirrored writes from x < 0 to x > 0).
__global__ void __launch_bounds__(256, 4)
k_insert_gather(float4* __restrict__ acc, int vdim, const float4* __restrict__ grid, int gw,
                int Rg, const float* __restrict__ rot, const float* __restrict__ tab, int tabNz,
                float tabInvStep, int pf, float Rp, float hs)
{
    const int dl = blockIdx.y;
    const float* mr = rot + 16 * (size_t)dl;
    const float e1x = __ldg(mr + 0), e1y = __ldg(mr + 3), e1z = __ldg(mr + 6);
    const float e2x = __ldg(mr + 1), e2y = __ldg(mr + 4), e2z = __ldg(mr + 7);
    const float e3x = __ldg(mr + 2), e3y = __ldg(mr + 5), e3z = __ldg(mr + 8);
    const float4* g = grid + (size_t)dl * gw * (2 * Rg + 1);
    const int half = vdim / 2, nx = half + 1;
    const float Rc = Rp + hs;                           // cylinder radius
    const float R2 = Rc * Rc + hs * hs;                 // |v|^2 bound
    const int Y = min(half - 1, (int)ceilf(Rc * sqrtf(fmaxf(0.f, 1.f - e3y * e3y)) +
                                           hs * fabsf(e3y)));
    const int Z = min(half - 1, (int)ceilf(Rc * sqrtf(fmaxf(0.f, 1.f - e3z * e3z)) +
                                           hs * fabsf(e3z)));
    const int ny = 2 * Y + 1;
    const int nRows = ny * (2 * Z + 1);
    const float fpf = (float)pf, inv_pf = 1.0f / fpf;

    for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < nRows;
         row += gridDim.x * blockDim.x) {
        const int y = row % ny - Y, z = row / ny - Z;
        const float fy = (float)y, fz = (float)z;
        const float rem = R2 - fy * fy - fz * fz;
        if (rem < 0.f) continue;
        const float hyz = e3y * fy + e3z * fz;
        float lo = 0.f, hi = fminf(sqrtf(rem), (float)(half - 1));
        if (fabsf(e3x) > 1e-6f) {
            const float ta = (-hs - hyz) / e3x, tb = (hs - hyz) / e3x;
            lo = fmaxf(lo, fminf(ta, tb));
            hi = fminf(hi, fmaxf(ta, tb));
        } else if (fabsf(hyz) > hs) {
            continue;
        }
        if (hi < lo) continue;
        const int xa = max((int)ceilf(lo - 1e-3f), 0);
        const int xb = min((int)floorf(hi + 1e-3f), half - 1);
        const float ayz = e1y * fy + e1z * fz, byz = e2y * fy + e2z * fz;
        float4* line = acc + ((size_t)(z < 0 ? z + vdim : z) * vdim + (y < 0 ? y + vdim : y)) * nx;
        for (int x = xa; x <= xb; x++) {
            const float fx = (float)x;
            const float a = fmaf(e1x, fx, ayz);
            const float b = fmaf(e2x, fx, byz);
            const float h = fmaf(e3x, fx, hyz);
            const float h2 = h * h;
            const int c0 = (int)ceilf((a - hs) * inv_pf), c1 = (int)floorf((a + hs) * inv_pf);
            const int q0 = max((int)ceilf((b - hs) * inv_pf), -Rg);
            const int q1 = min((int)floorf((b + hs) * inv_pf), Rg);
            float sr = 0.f, si = 0.f, st = 0.f;
            for (int c = c0; c <= c1; c++) {
                const float dx = a - fpf * (float)c;
                const float dx2h = fmaf(dx, dx, h2);
                for (int r = q0; r <= q1; r++) {
                    const float dy = b - fpf * (float)r;
                    const int ti = __float2int_rn(fmaf(dy, dy, dx2h) * tabInvStep);
                    if (ti > tabNz) continue;
                    const float kv = __ldg(tab + ti);
                    if (c >= 0 && c <= Rg) {
                        const float4 v = __ldg(g + (r + Rg) * gw + c);
                        sr = fmaf(kv, v.x, sr);
                        si = fmaf(kv, v.y, si);
                        st = fmaf(kv, v.z, st);
                    }
                    if (x > 0 && c <= 0 && -c <= Rg) {
                        const float4 v = __ldg(g + (Rg - r) * gw - c);
                        sr = fmaf(kv, v.x, sr);
                        si = fmaf(-kv, v.y, si);
                        st = fmaf(kv, v.z, st);
                    }
                }
            }
            if (sr != 0.f || si != 0.f || st != 0.f)
                atomicAdd(line + x, make_float4(sr, si, st, 0.f));
        }
    }
}

// ------------------------------------------------------------------------
// Projection banks: one class's projections at a fixed rotation set, made
// once (k_project) and gathered by index for every particle that uses them.
// Planes: hi = bf16(x), lo = bf16(x - hi), the rounding of the split store.
__global__ void k_bank_planes(const float* __restrict__ f32, int nB, int K, int Kp,
                              __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                              float* __restrict__ abs2)
{
    const size_t pairs = (size_t)nB * (Kp / 2);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / (Kp / 2);
        const int p = (int)(i % (Kp / 2));
        const float2 v = reinterpret_cast<const float2*>(f32 + row * Kp)[p];
        __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
        const float2 hf = __bfloat1622float2(h);
        reinterpret_cast<__nv_bfloat162*>(hi + row * Kp)[p] = h;
        reinterpret_cast<__nv_bfloat162*>(lo + row * Kp)[p] =
            __floats2bfloat162_rn(v.x - hf.x, v.y - hf.y);
        if (p < K) abs2[row * K + p] = v.x * v.x + v.y * v.y;
    }
}

// CTA (particle, group of 64 rows): w = sigRcp ctf^2 of the particle in
// shared memory; a warp per row copies the bank row in 16-byte units and
// sums its norm with shuffles.
constexpr int kBankRows = 64;

__global__ void __launch_bounds__(256)
k_bank_gather(const BankView* __restrict__ table, const int* __restrict__ cls,
              const int* __restrict__ idx, int nR, int K, int Kp,
              const float* __restrict__ sigRcp, const float* __restrict__ ctf,
              float* __restrict__ P, long long splitLo, float* __restrict__ nrm,
              int* __restrict__ flag)
{
    extern __shared__ float w[];                 // [K]
    const int l = blockIdx.x;
    const BankView b = table[cls ? cls[l] : 0];
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        const float c = ctf[(size_t)l * K + p];
        w[p] = sigRcp[(size_t)l * K + p] * c * c;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j1 = min(nR, (blockIdx.y + 1) * kBankRows);
    const int n16 = Kp / 4;                      // 16-byte units of a row (4 floats / 8 bf16)
    for (int j = blockIdx.y * kBankRows + warp; j < j1; j += 8) {
        const size_t row = (size_t)l * nR + j;
        const int r = idx[row];
        const bool ok = r >= 0 && r < b.nB;
        if (!ok && lane == 0) atomicOr(flag, 1 << 16);
        const size_t rs = (size_t)(ok ? r : 0);
        if (splitLo == 0) {
            const float4* src = reinterpret_cast<const float4*>(b.f32 + rs * Kp);
            float4* dst = reinterpret_cast<float4*>(P + row * Kp);
            for (int u = lane; u < n16; u += 32)
                dst[u] = ok ? __ldg(src + u) : make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            __nv_bfloat16* hp = reinterpret_cast<__nv_bfloat16*>(P);
            const uint4* sh = reinterpret_cast<const uint4*>(b.hi + rs * Kp);
            const uint4* sl = reinterpret_cast<const uint4*>(b.lo + rs * Kp);
            uint4* dh = reinterpret_cast<uint4*>(hp + row * Kp);
            uint4* dl = reinterpret_cast<uint4*>(hp + splitLo + row * Kp);
            const uint4 z = make_uint4(0u, 0u, 0u, 0u);
            for (int u = lane; u < n16 / 2; u += 32) {
                dh[u] = ok ? __ldg(sh + u) : z;
                dl[u] = ok ? __ldg(sl + u) : z;
            }
        }
        float acc = 0.f;
        if (ok) {
            const float* a2 = b.abs2 + rs * K;
            for (int p = lane; p < K; p += 32) acc = fmaf(w[p], __ldg(a2 + p), acc);
        }
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) nrm[row] = acc;
    }
}

// Fourier shell correlation of two half volumes [vdim][vdim][vdim/2+1] of
// complex values (FSC(vec&, const Volume&, const Volume&),
// src/Functions/Spectrum.cpp:302-329): shell u = rint(|k|) in voxel units,
// for u < nShell, of sum Re(A conj B), sum |A|^2, sum |B|^2 in FP64.  Each
// CTA sums its voxels per shell in shared memory, then adds its shells once.
__global__ void __launch_bounds__(256)
k_fsc_shells(const float2* __restrict__ A, const float2* __restrict__ B, int vdim, int nShell,
             double* __restrict__ sums)
{
    extern __shared__ double sacc[];             // [3][nShell]
    for (int i = threadIdx.x; i < 3 * nShell; i += blockDim.x) sacc[i] = 0.0;
    __syncthreads();
    const int nx = vdim / 2 + 1, half = vdim / 2;
    const size_t n = (size_t)vdim * vdim * nx;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx);
        const size_t zy = i / nx;
        const int y = (int)(zy % vdim), z = (int)(zy / vdim);
        const int fy = y < half ? y : y - vdim, fz = z < half ? z : z - vdim;
        const int u = __double2int_rn(sqrt((double)x * x + (double)fy * fy + (double)fz * fz));
        if (u >= nShell) continue;
        const float2 a = A[i], b = B[i];
        atomicAdd(sacc + u, (double)a.x * b.x + (double)a.y * b.y);
        atomicAdd(sacc + nShell + u, (double)a.x * a.x + (double)a.y * a.y);
        atomicAdd(sacc + 2 * nShell + u, (double)b.x * b.x + (double)b.y * b.y);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * nShell; i += blockDim.x)
        if (sacc[i] != 0.0) atomicAdd(sums + i, sacc[i]);
}

__global__ void k_fsc_finish(const double* __restrict__ sums, int nShell, double* __restrict__ fsc)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nShell) return;
    const double xy = sums[u], xx = sums[nShell + u], yy = sums[2 * nShell + u];
    fsc[u] = (xx * yy == 0.0) ? 0.0 : xy / sqrt(xx * yy);
}

// V = F / T where T > floor, else 0: the inserted slices' average at every
// voxel of the accumulator.
__global__ void k_acc_ratio(const float4* __restrict__ acc, size_t n, float floor_,
                            float2* __restrict__ V)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        V[i] = a.z > floor_ ? make_float2(a.x / a.z, a.y / a.z) : make_float2(0.f, 0.f);
    }
}

__global__ void k_acc_read(const float4* __restrict__ acc, size_t n, float2* __restrict__ F,
                           float* __restrict__ T, int accumulate)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float4 a = acc[i];
        if (accumulate) {
            float2 f = F[i];
            F[i] = make_float2(f.x + a.x, f.y + a.y);
            T[i] += a.z;
        } else {
            F[i] = make_float2(a.x, a.y);
            T[i] = a.z;
        }
    }
}

inline int grid_for(size_t n, int block, int cap = 152 * 16)
{
    size_t g = (n + block - 1) / block;
    if (g > (size_t)cap) g = cap;
    return (int)(g ? g : 1);
}

}  // namespace

// ---------------------------------------------------------------- launchers
cudaError_t launch_rotmat(const double* quat, int n, double* mat, cudaStream_t st)
{
    k_rotmat<<<(n + 127) / 128, 128, 0, st>>>(quat, n, mat);
    return cudaGetLastError();
}

cudaError_t launch_translate(const double* trans, int nT, int idim, const int* iCol,
                             const int* iRow, int K, float2* out, int ldo2, cudaStream_t st)
{
    dim3 grid((ldo2 + 255) / 256, nT);
    k_translate<<<grid, 256, 0, st>>>(trans, nT, idim, iCol, iRow, K, out, ldo2);
    return cudaGetLastError();
}

cudaError_t launch_ctf(const float* attr, int nImg, float px, int idim, const int* iCol,
                       const int* iRow, int K, float* out, cudaStream_t st)
{
    dim3 grid(nImg);
    k_ctf<<<grid, 256, 0, st>>>(attr, nImg, px, idim, iCol, iRow, K, out);
    return cudaGetLastError();
}

size_t volume_block_count(int vdim)
{
    return (size_t)cubes_x(vdim) * cubes_yz(vdim) * cubes_yz(vdim) * 32768;
}

cudaError_t launch_volume_blocks(const float2* vol, int vdim, float4* blocks, cudaStream_t st)
{
    size_t n = (size_t)vdim * vdim * (vdim / 2 + 1);
    k_volume_blocks<<<grid_for(n, 256), 256, 0, st>>>(vol, vdim, blocks);
    return cudaGetLastError();
}

cudaError_t launch_rot_f32(const double* quat, const double* mat, int rows, float* mf,
                           cudaStream_t st)
{
    if (rows <= 0) return cudaSuccess;
    k_rot_f32<<<grid_for((size_t)rows, 256), 256, 0, st>>>(quat, mat, rows, mf);
    return cudaGetLastError();
}

int project_chunks(int ldo) { return (ldo / 2 + kProjChunk - 1) / kProjChunk; }

size_t project_scratch_floats(int rows, int ldo)
{
    return (size_t)rows * (9 + project_chunks(ldo));
}

cudaError_t launch_project(float4* const* volTable, const int* cls, const float4* vol,
                           int vdim, int pf, const double* quat, const double* mat,
                           int rows, int rowsPerParticle, const int* iCol,
                           const int* iRow, int K, float* out, int ldo,
                           const float* sigRcp, const float* ctf, float* nrm, float* scratch,
                           int* flag, long long splitLo, cudaStream_t st, int form, int group)
{
    if (rows <= 0) return cudaSuccess;
    if (!scratch || rows % rowsPerParticle) return cudaErrorInvalidValue;
    static_assert(kProjChunk % 256 == 0, "one lane per pixel takes whole 256-pixel passes");
    const int nP = rows / rowsPerParticle;
    if (group != 4 && group != 8 && group != 16) return cudaErrorInvalidValue;
    // the rotation group of a CTA: kProjG for forms 0 - 2, `group` for 3 and 4
    const int G = form >= 3 ? group : kProjG;
    const int nGroups = (rowsPerParticle + G - 1) / G;
    const int nChunks = project_chunks(ldo);
    const long long grid = (long long)nP * nChunks * nGroups;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    float* mf = scratch;
    float* nrmPart = scratch + (size_t)rows * 9;
    k_rot_f32<<<grid_for((size_t)rows, 256), 256, 0, st>>>(quat, mat, rows, mf);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t tabBytes = sizeof(int) * ((size_t)vdim / 2 + 1 + 2 * (size_t)vdim);
    auto kern = form == 4   ? (G == 4 ? k_project_xchg<true, 4> : G == 16 ? k_project_xchg<true, 16>
                                                                   : k_project_xchg<true, 8>)
                : form == 3 ? (G == 4 ? k_project_xchg<false, 4> : G == 16 ? k_project_xchg<false, 16>
                                                                    : k_project_xchg<false, 8>)
                : form == 2 ? k_project_lane<true>
                : form == 1 ? k_project_lane<false>
                            : k_project;
    if (tabBytes > 48 * 1024) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tabBytes);
        if (e != cudaSuccess) return e;
    }
    kern<<<(unsigned)grid, 256, tabBytes, st>>>(volTable, cls, vol, vdim, pf, mf, rowsPerParticle,
                                                nGroups, nChunks, iCol, iRow, K, out, ldo, sigRcp,
                                                ctf, nrm ? nrmPart : nullptr, flag, splitLo);
    e = cudaGetLastError();
    if (e != cudaSuccess || !nrm) return e;
    k_norm_reduce<<<grid_for((size_t)rows, 256), 256, 0, st>>>(nrmPart, rows, nChunks, nrm);
    return cudaGetLastError();
}

cudaError_t launch_shift_bank(const float2* dat, const float* ctf, const float* sigRcp,
                              const double* trans, const float2* bank, int nP, int nT,
                              int idim, const int* iCol, const int* iRow, int K, float* out,
                              int ldo, long long splitLo, cudaStream_t st, int nD)
{
    if (nD < 1 || nT < 1) return cudaErrorInvalidValue;
    // groups of at most SHIFT_T translations, as even as possible (25 as
    // 7 + 7 + 7 + 4, not 8 + 8 + 8 + 1: every CTA reloads its pixels)
    const int groups = (nT + SHIFT_T - 1) / SHIFT_T;
    const int tPer = (nT + groups - 1) / groups;
    dim3 grid((unsigned)nP * nD, (nT + tPer - 1) / tPer);
    // the separable phase tables when they fit the default shared memory
    const size_t tab = bank ? 0 : sizeof(float2) * SHIFT_T * (size_t)(3 * (idim / 2) + 2);
    const int useTab = (!bank && idim >= 2 && tab <= 48 * 1024) ? 1 : 0;
    k_shift_bank<<<grid, 256, useTab ? tab : 0, st>>>(dat, ctf, sigRcp, trans, bank, nT, nD, idim,
                                                      iCol, iRow, K, out, ldo, splitLo, useTab,
                                                      tPer);
    return cudaGetLastError();
}

cudaError_t launch_norm_defocus(const float* P, long long splitLo, int nP, int nR, int nD, int K,
                                int Kp, const float* sigRcp, const float* ctf, float* nrm,
                                cudaStream_t st)
{
    if (nD < 1 || nD > kMaxDefocus) return cudaErrorInvalidValue;
    k_norm_defocus<<<dim3(nP, (nR + 7) / 8), 256, 0, st>>>(P, splitLo, nP, nR, nD, K, Kp, sigRcp,
                                                           ctf, nrm);
    return cudaGetLastError();
}

cudaError_t launch_project2d(const float2* img, int vdim, int pf, const double* rot, int nR,
                             const int* iCol, const int* iRow, int K, float* out, int ldo,
                             long long splitLo, cudaStream_t st)
{
    if (nR <= 0 || nR > 65535) return cudaErrorInvalidValue;
    k_project2d<<<dim3((ldo / 2 + 255) / 256, nR), 256, 0, st>>>(img, vdim, pf, rot, iCol, iRow,
                                                                K, out, ldo, splitLo);
    return cudaGetLastError();
}

cudaError_t launch_insert2d(float4* acc, int vdim, const float2* dat, const float* ctf,
                            int ctfPerDraw, const float* w, const double* offS, const int* nC,
                            const double* nR, const double* nT, const int* iCol, const int* iRow,
                            int K, int pf, int idim, int nDraws, int drawsPerImage, double* O2D,
                            int* counter, cudaStream_t st)
{
    const int tiles = std::max(1, std::min(1024, (K + 255) / 256));
    for (int d0 = 0; d0 < nDraws; d0 += 65535) {
        const int n = std::min(65535, nDraws - d0);
        k_insert2d<<<dim3(tiles, n), 256, 0, st>>>(acc, vdim, dat, ctf, ctfPerDraw, w, offS, nC, nR,
                                                   nT, iCol, iRow, K, pf, idim, d0,
                                                   drawsPerImage, O2D, counter);
    }
    return cudaGetLastError();
}

cudaError_t launch_draw_attr(const float* attr, const double* nD, int nDraws, int drawsPerImage,
                             float* out, cudaStream_t st)
{
    k_draw_attr<<<(nDraws + 255) / 256, 256, 0, st>>>(attr, nD, nDraws, drawsPerImage, out);
    return cudaGetLastError();
}

cudaError_t launch_ctf_defocus(const float* defO, const float* freQ, const double* dpara, int nD,
                               int K, double k1, double k2, double phaseShift, double conT,
                               float* ctf, cudaStream_t st)
{
    k_ctf_defocus<<<dim3((K + 255) / 256, nD), 256, 0, st>>>(defO, freQ, dpara, K, k1, k2,
                                                            phaseShift, conT, ctf);
    return cudaGetLastError();
}

cudaError_t launch_repeat_rows(const double* src, int rows, int len, int nRep, double* dst,
                               cudaStream_t st)
{
    k_repeat_rows<<<grid_for((size_t)rows * nRep * len, 256), 256, 0, st>>>(src, rows, len, nRep,
                                                                          dst);
    return cudaGetLastError();
}

cudaError_t launch_merge_defocus(int nP, int nD, int nR, int nT, const double* wCb,
                                 const double* wRb, const double* wTb, const double* baseb,
                                 const double* pwD, double* wC, double* wR, double* wT,
                                 double* wD, double* base, cudaStream_t st)
{
    if (nD < 1 || nD > kMaxDefocus) return cudaErrorInvalidValue;
    k_merge_defocus<<<nP, 256, 0, st>>>(nD, nR, nT, wCb, wRb, wTb, baseb, pwD, wC, wR, wT, wD,
                                        base);
    return cudaGetLastError();
}

cudaError_t launch_x0(const float2* dat, const float* sigRcp, int nP, int K, double* x0,
                      cudaStream_t st)
{
    k_x0<<<nP, 256, 0, st>>>(dat, sigRcp, K, x0);
    return cudaGetLastError();
}

cudaError_t launch_gemm_nt_fp32(const float* A, long long sA, int lda, const float* B,
                                long long sB, int ldb, int M, int N, int Kd, int batch,
                                float* C, long long sC, int ldc, const float* nrm,
                                long long sN, float alpha, cudaStream_t st, int cGroup,
                                long long cGroupStride)
{
    dim3 grid((N + GB_N - 1) / GB_N, (M + GB_M - 1) / GB_M, batch);
    k_gemm_nt_fp32<<<grid, 256, 0, st>>>(A, sA, lda, B, sB, ldb, M, N, Kd, C, sC, ldc,
                                          nrm, sN, alpha, cGroup, cGroupStride);
    return cudaGetLastError();
}

// out[i] = sum over the S partial results part[b][i], b = 0 .. S-1 in order
// (the split-K chunks of a GEMM).
__global__ void k_sum_parts(const float* __restrict__ part, int S, size_t cnt,
                            float* __restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < cnt;
         i += (size_t)gridDim.x * blockDim.x) {
        float v = part[i];
        for (int b = 1; b < S; b++) v += part[(size_t)b * cnt + i];
        out[i] = v;
    }
}

cudaError_t launch_sum_parts(const float* part, int S, size_t cnt, float* out, cudaStream_t st)
{
    if (S < 1) return cudaErrorInvalidValue;
    const unsigned blocks = (unsigned)std::min<size_t>((cnt + 255) / 256, 152 * 16);
    k_sum_parts<<<blocks, 256, 0, st>>>(part, S, cnt, out);
    return cudaGetLastError();
}

// Fold the row chunks of k_weights (nc per item): M = max_c base_c, every
// chunk scaled by exp(base_c - M): wC, wT summed over the chunks in order, the
// chunk's wR rows rescaled in place, base = M.  One CTA per item.
__global__ void k_merge_chunks(int nc, int nR, int nT, const double* __restrict__ wCc,
                               const double* __restrict__ wTc, const double* __restrict__ basec,
                               double* __restrict__ wC, double* __restrict__ wR,
                               double* __restrict__ wT, double* __restrict__ base)
{
    extern __shared__ double sc[];   // [nc]
    const int l = blockIdx.x;
    const double* bc = basec + (size_t)l * nc;
    double M = bc[0];
    for (int c = 1; c < nc; c++) M = fmax(M, bc[c]);
    for (int c = threadIdx.x; c < nc; c += blockDim.x) sc[c] = exp(bc[c] - M);
    __syncthreads();
    const int rpb = (nR + nc - 1) / nc;
    for (int r = threadIdx.x; r < nR; r += blockDim.x) wR[(size_t)l * nR + r] *= sc[r / rpb];
    for (int t = threadIdx.x; t < nT; t += blockDim.x) {
        double v = 0.0;
        for (int c = 0; c < nc; c++) v += wTc[((size_t)l * nc + c) * nT + t] * sc[c];
        wT[(size_t)l * nT + t] = v;
    }
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int c = 0; c < nc; c++) v += wCc[(size_t)l * nc + c] * sc[c];
        wC[l] = v;
        base[l] = M;
    }
}

cudaError_t launch_weights(const float* D, long long sD, int ldc, int nR, int nT, int G,
                           int nBlocks, const float* nrmG, int nrmRS, const double* x0,
                           const double* pwR,
                           long long sR, const double* pwT, long long sT, const double* pwC,
                           double* wC, double* wR, double* wT, double* base, float* dvp,
                           cudaStream_t st, int threads, int nc, double* chunkTmp)
{
    if (nc < 1 || (nc > 1 && (G != 1 || !chunkTmp))) return cudaErrorInvalidValue;
    if (threads != 128 && threads != 256 && threads != WEIGHTS_THREADS)
        return cudaErrorInvalidValue;
    const size_t smem = sizeof(float) * (2 + (nT <= 256 ? threads / 32 : 0)) * (size_t)nT;
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    // nc > 1: per-chunk wC, wT, base in chunkTmp, folded afterwards
    double* cC = nc > 1 ? chunkTmp : wC;
    double* cB = nc > 1 ? chunkTmp + (size_t)nBlocks * nc : base;
    double* cT = nc > 1 ? chunkTmp + 2 * (size_t)nBlocks * nc : wT;
#define TG3_WEIGHTS(TS)                                                                        \
    k_weights<TS><<<nBlocks * nc, threads, smem, st>>>(D, sD, ldc, nR, nT, G, nrmG, nrmRS, x0, \
                                                       pwR, sR, pwT, sT, pwC, cC, wR, cT, cB,  \
                                                       dvp, nc)
    if (nT <= 32) TG3_WEIGHTS(1);
    else if (nT <= 64) TG3_WEIGHTS(2);
    else if (nT <= 128) TG3_WEIGHTS(4);
    else if (nT <= 256) TG3_WEIGHTS(8);
    else TG3_WEIGHTS(0);
#undef TG3_WEIGHTS
    if (nc > 1) {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_merge_chunks<<<nBlocks, 128, sizeof(double) * nc, st>>>(nc, nR, nT, cC, cT, cB, wC, wR,
                                                                  wT, base);
    }
    return cudaGetLastError();
}

cudaError_t launch_merge_class(int nImg, int nK, int kIdx, int nR, int nT, const double* wCn,
                               const double* wRn, const double* wTn, const double* basen,
                               float* wC, float* wR, float* wT, float* baseL, cudaStream_t st,
                               int inStride)
{
    k_merge_class<<<nImg, 256, 0, st>>>(nK, kIdx, nR, nT, wCn, wRn, wTn, basen, wC, wR, wT,
                                         baseL, inStride);
    return cudaGetLastError();
}

// All nK per-(image, class) weight blocks of a multi-class scan folded into
// ExpectGlobal2D's outputs in one pass: relative to the image's best class,
// class k scaled by exp(base_k - max_k base_k) -- the value the running
// baseline of kernel_setBaseLine / kernel_UpdateW reaches class by class.
// One CTA per image; smem: nK doubles.
__global__ void k_merge_classes(int nK, int nR, int nT, const double* __restrict__ wCn,
                                const double* __restrict__ wRn, const double* __restrict__ wTn,
                                const double* __restrict__ basen, float* __restrict__ wC,
                                float* __restrict__ wR, float* __restrict__ wT,
                                float* __restrict__ baseL)
{
    extern __shared__ double esc[];
    __shared__ double Bm;
    const size_t l = blockIdx.x;
    const double* bl = basen + l * nK;
    if (threadIdx.x == 0) {
        double m = bl[0];
        for (int k = 1; k < nK; k++) m = fmax(m, bl[k]);
        Bm = m;
        baseL[l] = (float)m;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nK; k += blockDim.x) {
        esc[k] = exp(bl[k] - Bm);
        wC[l * nK + k] = (float)(wCn[l * nK + k] * esc[k]);
    }
    __syncthreads();
    const size_t oR = l * nK * nR, oT = l * nK * nT;
    for (int i = threadIdx.x; i < nK * nR; i += blockDim.x)
        wR[oR + i] = (float)(wRn[oR + i] * esc[i / nR]);
    for (int i = threadIdx.x; i < nK * nT; i += blockDim.x)
        wT[oT + i] = (float)(wTn[oT + i] * esc[i / nT]);
}

cudaError_t launch_merge_classes(int nImg, int nK, int nR, int nT, const double* wCn,
                                 const double* wRn, const double* wTn, const double* basen,
                                 float* wC, float* wR, float* wT, float* baseL, cudaStream_t st)
{
    const size_t smem = sizeof(double) * (size_t)nK;
    if (smem > 48 * 1024) return cudaErrorInvalidValue;
    k_merge_classes<<<nImg, 256, smem, st>>>(nK, nR, nT, wCn, wRn, wTn, basen, wC, wR, wT, baseL);
    return cudaGetLastError();
}

__global__ void k_nrm_classes(const float* __restrict__ nrm, int nK, int nR, int n,
                              float* __restrict__ out)
{
    const size_t total = (size_t)nK * nR * n;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        // i walks the output: i = r (n nK) + l nK + k
        const int k = (int)(i % nK);
        const size_t rl = i / nK;
        const int l = (int)(rl % n);
        const int r = (int)(rl / n);
        out[i] = nrm[((size_t)k * nR + r) * n + l];
    }
}

cudaError_t launch_nrm_classes(const float* nrm, int nK, int nR, int n, float* out,
                               cudaStream_t st)
{
    k_nrm_classes<<<grid_for((size_t)nK * nR * n, 256), 256, 0, st>>>(nrm, nK, nR, n, out);
    return cudaGetLastError();
}

cudaError_t launch_resample(int nP, int n, const double* u, const double* w, const int* perm,
                            const double* u0, const double* peak, int nOut, int* src,
                            double* wOut, int* top, int* flag, cudaStream_t st, const int* nPer)
{
    size_t smem = sizeof(double) * (2 * (size_t)n + (size_t)(n > nOut ? n : nOut))
                + sizeof(int) * (size_t)n;
    cudaError_t e = cudaFuncSetAttribute(k_resample, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    k_resample<<<nP, 256, smem, st>>>(n, u, w, perm, u0, peak, nOut, nPer, src, wOut, top, flag);
    return cudaGetLastError();
}

cudaError_t launch_insert(float4* acc, int vdim, int kernel, const float* tab, int tabNz,
                          float tabInvStep, int nDraws, int drawsPerImage, const float2* dat,
                          const float* ctf, const double* quat, const double* trans,
                          const double* offset, const float* w, const int* iCol,
                          const int* iRow, int K, int pf, int idim, double* O3D, int* counter,
                          float* params, cudaStream_t st, int ctfRows, const int* nC)
{
    if (nDraws <= 0) return cudaSuccess;
    // r^2 bound of the table's support: rint(r^2 n / b) <= tabNz  =>  r^2 < (tabNz + 1/2) b / n
    const float rs2 = (((float)tabNz + 0.5f) / tabInvStep) * (1.0f + 1e-4f);
    if (kernel == TG3_KERNEL_MKB && 2.0f * sqrtf(rs2) >= 4.0f) return cudaErrorInvalidValue;
    k_insert_draws<<<(nDraws + 255) / 256, 256, 0, st>>>(nDraws, drawsPerImage, quat, trans,
                                                         offset, w, params, O3D, counter, nC);
    const int ctfPerDraw = ctfRows == nDraws && drawsPerImage > 1;
    // one pixel per thread: the draw's pixels spread over ceil(K / 256) CTAs
    const int tiles = std::max(1, std::min(1024, (K + 255) / 256));
    for (int d0 = 0; d0 < nDraws; d0 += 65535) {
        const int n = std::min(65535, nDraws - d0);
        k_insert<<<dim3(tiles, n), 256, 0, st>>>(acc, vdim, kernel, tab, tabNz, tabInvStep, rs2,
                                                 dat, ctf, params, iCol, iRow, K, pf, idim, d0,
                                                 drawsPerImage, ctfPerDraw);
    }
    return cudaGetLastError();
}

size_t insert_draw_bytes(int Rg)
{
    return (size_t)(Rg + 1) * (2 * Rg + 1) * sizeof(float4) + 16 * sizeof(float);
}

cudaError_t launch_insert_gather(float4* acc, int vdim, const float* tab, int tabNz,
                                 float tabInvStep, int nDraws, int drawsPerImage,
                                 const float2* dat, const float* ctf, const double* quat,
                                 const double* trans, const double* offset, const float* w,
                                 const int* cellPix, const int* iCol, const int* iRow, int K,
                                 int pf, int idim, int Rg, float Rp, double* O3D, int* counter,
                                 void* scratch, size_t scratchBytes, cudaStream_t st, int ctfRows)
{
    if (nDraws <= 0) return cudaSuccess;
    const int ctfPerDraw = ctfRows == nDraws && drawsPerImage > 1;
    const int gw = Rg + 1, cells = gw * (2 * Rg + 1);
    const size_t gridBytes = (size_t)cells * sizeof(float4);
    const size_t chunkMax = scratchBytes / insert_draw_bytes(Rg);
    if (chunkMax < 1) return cudaErrorInvalidValue;
    const int chunk = (int)std::min<size_t>(std::min<size_t>((size_t)nDraws, chunkMax), 65535);
    float4* grid = static_cast<float4*>(scratch);
    float* rot = reinterpret_cast<float*>(static_cast<char*>(scratch) + gridBytes * chunk);
    // slab half thickness: rint(r^2 n / b) <= tabNz  <=>  r^2 < (tabNz + 1/2) b / n
    const float hs = sqrtf(((float)tabNz + 0.5f) / tabInvStep) + 1e-3f;
    const int stageTiles = std::max(1, std::min(64, (cells + 1023) / 1024));
    for (int d0 = 0; d0 < nDraws; d0 += chunk) {
        const int n = std::min(chunk, nDraws - d0);
        k_insert_stage<<<dim3(stageTiles, n), 256, 0, st>>>(grid, cells, rot, cellPix, iCol, iRow,
                                                            dat, ctf, quat, trans, offset, w, K,
                                                            idim, d0, drawsPerImage, ctfPerDraw,
                                                            O3D, counter);
        // about two waves of resident CTAs (152 SMs x 8 CTAs of 256 threads)
        const int tiles = std::max(1, std::min(128, (2 * 152 * 8 + n - 1) / n));
        k_insert_gather<<<dim3(tiles, n), 256, 0, st>>>(acc, vdim, grid, gw, Rg, rot, tab, tabNz,
                                                        tabInvStep, pf, Rp, hs);
    }
    return cudaGetLastError();
}

cudaError_t launch_bank_planes(const float* f32, int nB, int K, int Kp, __nv_bfloat16* hi,
                               __nv_bfloat16* lo, float* abs2, cudaStream_t st)
{
    k_bank_planes<<<grid_for((size_t)nB * (Kp / 2), 256), 256, 0, st>>>(f32, nB, K, Kp, hi, lo,
                                                                       abs2);
    return cudaGetLastError();
}

cudaError_t launch_bank_gather(const BankView* table, const int* cls, const int* idx, int nP,
                               int nR, int K, int Kp, const float* sigRcp, const float* ctf,
                               float* P, long long splitLo, float* nrm, int* flag,
                               cudaStream_t st)
{
    if (Kp % 8) return cudaErrorInvalidValue;
    const size_t smem = sizeof(float) * (size_t)K;
    if (smem > 48 * 1024) {
        if (smem > 200 * 1024) return cudaErrorInvalidValue;
        cudaError_t e = cudaFuncSetAttribute(k_bank_gather,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(nP, (nR + kBankRows - 1) / kBankRows);
    k_bank_gather<<<grid, 256, smem, st>>>(table, cls, idx, nR, K, Kp, sigRcp, ctf, P, splitLo,
                                           nrm, flag);
    return cudaGetLastError();
}

cudaError_t launch_fsc(const float2* A, const float2* B, int vdim, int nShell, double* sums,
                       double* fsc, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(sums, 0, sizeof(double) * 3 * (size_t)nShell, st);
    if (e != cudaSuccess) return e;
    const size_t smem = sizeof(double) * 3 * (size_t)nShell;
    e = cudaFuncSetAttribute(k_fsc_shells, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const size_t n = (size_t)vdim * vdim * (vdim / 2 + 1);
    k_fsc_shells<<<grid_for(n, 256, 152 * 4), 256, smem, st>>>(A, B, vdim, nShell, sums);
    k_fsc_finish<<<(nShell + 127) / 128, 128, 0, st>>>(sums, nShell, fsc);
    return cudaGetLastError();
}

cudaError_t launch_acc_ratio(const float4* acc, size_t n, float floor_, float2* V, cudaStream_t st)
{
    k_acc_ratio<<<grid_for(n, 256), 256, 0, st>>>(acc, n, floor_, V);
    return cudaGetLastError();
}

cudaError_t launch_acc_read(const float4* acc, size_t n, float2* F, float* T, int accumulate,
                            cudaStream_t st)
{
    k_acc_read<<<grid_for(n, 256), 256, 0, st>>>(acc, n, F, T, accumulate);
    return cudaGetLastError();
}

}  // namespace tg3
