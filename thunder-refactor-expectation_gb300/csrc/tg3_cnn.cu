// tg3_cnn.cu -- the pose-proposal network: forward, backward and Adam, all
// hand-written kernels (no library calls).
//
// Input: a 64 x 64 particle image (real space, normalised).  Layers:
//   conv1  1 -> 32, 3x3, stride 1   64 x 64
//   conv2 32 -> 32, 3x3, stride 2   32 x 32
//   conv3 32 -> 64, stride 1        32 x 32
//   conv4 64 -> 64, stride 2        16 x 16
//   conv5 64 -> 128, stride 1       16 x 16
//   conv6 128 -> 128, stride 2       8 x  8     (every conv: pad 1, bias, ReLU)
//   fc1  8192 -> 256, ReLU;  fc2  256 -> 68.
// Output per image: 8 mixture components x (6-D rotation, raw concentration,
// logit) = 64 values, then the shift mean (2) and its log-variance (2).
// The weights are used in bf16 (rounded from FP32 master copies on every
// load), activations and accumulation are FP32.
//
// Loss per image (the negative log-likelihood of the true pose):
//   R_k = GramSchmidt(a_k, b_k),  c_k = (tr(R_k^T R*) - 1) / 2 = cos(angle),
//   kappa_k = softplus(raw_k) + 1e-3,
//   -log sum_k softmax(logit)_k kappa_k^{3/2} exp(kappa_k (c_k - 1))
//   + 0.5 sum_d ((t*_d - mu_d)^2 exp(-lv_d) + lv_d).
// (A concentrated rotation density in the angle: kappa^{3/2} exp(-kappa
// angle^2 / 2) for small angles, up to constants.)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {

namespace {

constexpr int kLayers = 8;   // 6 conv + 2 fc

inline int cnn_grid(size_t n, int block)
{
    const size_t g = (n + block - 1) / block;
    return (int)(g < 4096 ? (g ? g : 1) : 4096);
}
constexpr int kOut = 68;
constexpr int kComp = 8;

struct LayerShape {
    int cin, cout, hin, hout, stride;   // fc: hin = hout = 1, stride 0
};

constexpr LayerShape kShape[kLayers] = {
    {1, 32, 64, 64, 1},   {32, 32, 64, 32, 2},  {32, 64, 32, 32, 1},  {64, 64, 32, 16, 2},
    {64, 128, 16, 16, 1}, {128, 128, 16, 8, 2}, {8192, 256, 1, 1, 0}, {256, kOut, 1, 1, 0}};

__host__ __device__ inline size_t weight_count(const LayerShape& s)
{
    return s.stride ? (size_t)s.cout * s.cin * 9 : (size_t)s.cout * s.cin;
}

// weights as the forward and backward passes use them: rounded to bf16, or
// kept in FP32 (gradient checks by finite differences need a smooth loss)
__device__ __forceinline__ float bf(float w, int round = 1)
{
    return round ? __bfloat162float(__float2bfloat16_rn(w)) : w;
}

// ---------------------------------------------------------------- conv ---
// y[n][co][oy][ox] = relu(b[co] + sum_ci,ky,kx W[co][ci][ky][kx] x[n][ci][oy s + ky - 1][ox s + kx - 1])
// CTA: 16 output channels x 256 output pixels of one image; weights of a
// 16-channel input slice staged in shared memory.
__global__ void __launch_bounds__(256)
k_conv_fwd(const float* __restrict__ x, const float* __restrict__ W, const float* __restrict__ b,
           float* __restrict__ y, int cin, int cout, int hin, int hout, int stride, int relu,
           int roundW)
{
    __shared__ float ws[16][16][9];
    const int n = blockIdx.z, co0 = blockIdx.y * 16;
    const int pix = blockIdx.x * 256 + threadIdx.x;
    const int oy = pix / hout, ox = pix % hout;
    const bool valid = pix < hout * hout;
    float acc[16];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] = 0.f;
    const float* xn = x + (size_t)n * cin * hin * hin;
    for (int ci0 = 0; ci0 < cin; ci0 += 16) {
        __syncthreads();
        for (int i = threadIdx.x; i < 16 * 16 * 9; i += 256) {
            const int c = i / 144, cc = (i / 9) % 16, k = i % 9;
            ws[c][cc][k] = (co0 + c < cout && ci0 + cc < cin)
                               ? bf(W[((size_t)(co0 + c) * cin + ci0 + cc) * 9 + k], roundW)
                               : 0.f;
        }
        __syncthreads();
        if (!valid) continue;
        const int ncc = min(16, cin - ci0);
        for (int cc = 0; cc < ncc; cc++) {
            const float* xc = xn + (size_t)(ci0 + cc) * hin * hin;
            float v[9];
#pragma unroll
            for (int ky = 0; ky < 3; ky++)
#pragma unroll
                for (int kx = 0; kx < 3; kx++) {
                    const int iy = oy * stride + ky - 1, ix = ox * stride + kx - 1;
                    v[ky * 3 + kx] = (iy >= 0 && iy < hin && ix >= 0 && ix < hin) ? xc[iy * hin + ix] : 0.f;
                }
#pragma unroll
            for (int c = 0; c < 16; c++)
#pragma unroll
                for (int k = 0; k < 9; k++) acc[c] = fmaf(ws[c][cc][k], v[k], acc[c]);
        }
    }
    if (!valid) return;
    for (int c = 0; c < 16 && co0 + c < cout; c++) {
        float o = acc[c] + b[co0 + c];
        if (relu) o = fmaxf(o, 0.f);
        y[(((size_t)n * cout + co0 + c) * hout + oy) * hout + ox] = o;
    }
}

// dx[n][ci][iy][ix] = sum_co,ky,kx W[co][ci][ky][kx] dy[n][co][oy][ox] with
// iy = oy s + ky - 1 (the taps that reached the input pixel).  CTA: 16 input
// channels x 256 input pixels of one image.
__global__ void __launch_bounds__(256)
k_conv_bwd_data(const float* __restrict__ dy, const float* __restrict__ W, float* __restrict__ dx,
                int cin, int cout, int hin, int hout, int stride, int roundW)
{
    __shared__ float ws[16][16][9];   // [co slice][ci][k]
    const int n = blockIdx.z, ci0 = blockIdx.y * 16;
    const int pix = blockIdx.x * 256 + threadIdx.x;
    const int iy = pix / hin, ix = pix % hin;
    const bool valid = pix < hin * hin;
    float acc[16];
#pragma unroll
    for (int c = 0; c < 16; c++) acc[c] = 0.f;
    const float* dyn = dy + (size_t)n * cout * hout * hout;
    for (int co0 = 0; co0 < cout; co0 += 16) {
        __syncthreads();
        for (int i = threadIdx.x; i < 16 * 16 * 9; i += 256) {
            const int c = i / 144, cc = (i / 9) % 16, k = i % 9;
            ws[c][cc][k] = (co0 + c < cout && ci0 + cc < cin)
                               ? bf(W[((size_t)(co0 + c) * cin + ci0 + cc) * 9 + k], roundW)
                               : 0.f;
        }
        __syncthreads();
        if (!valid) continue;
        const int nc = min(16, cout - co0);
        for (int c = 0; c < nc; c++) {
            const float* dc = dyn + (size_t)(co0 + c) * hout * hout;
#pragma unroll
            for (int ky = 0; ky < 3; ky++) {
                const int ty = iy + 1 - ky;
                if (ty < 0 || ty % stride) continue;
                const int oy = ty / stride;
                if (oy >= hout) continue;
#pragma unroll
                for (int kx = 0; kx < 3; kx++) {
                    const int tx = ix + 1 - kx;
                    if (tx < 0 || tx % stride) continue;
                    const int ox = tx / stride;
                    if (ox >= hout) continue;
                    const float g = dc[oy * hout + ox];
#pragma unroll
                    for (int cc = 0; cc < 16; cc++) acc[cc] = fmaf(ws[c][cc][ky * 3 + kx], g, acc[cc]);
                }
            }
        }
    }
    if (!valid) return;
    for (int cc = 0; cc < 16 && ci0 + cc < cin; cc++)
        dx[(((size_t)n * cin + ci0 + cc) * hin + iy) * hin + ix] = acc[cc];
}

// dW[co][ci][k] += sum_n,oy,ox dy[n][co][oy][ox] x[n][ci][tap k], db[co] +=
// sum dy.  CTA: one output channel, 8 input channels, one slice of images;
// the CTA's partial sums go to the gradient with one atomic add each.
__global__ void __launch_bounds__(256)
k_conv_bwd_weight(const float* __restrict__ x, const float* __restrict__ dy, float* __restrict__ dW,
                  float* __restrict__ db, int N, int cin, int cout, int hin, int hout, int stride,
                  int imgPerCta)
{
    __shared__ float red[72 + 1][8];
    const int co = blockIdx.x, ci0 = blockIdx.y * 8, n0 = blockIdx.z * imgPerCta;
    const int nci = min(8, cin - ci0);
    float acc[8][9];
    float accb = 0.f;
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
        for (int k = 0; k < 9; k++) acc[c][k] = 0.f;
    const int P = hout * hout;
    const int total = min(imgPerCta, N - n0) * P;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        const int n = n0 + e / P, pix = e % P;
        const int oy = pix / hout, ox = pix % hout;
        const float g = dy[(((size_t)n * cout + co) * hout + oy) * hout + ox];
        if (g == 0.f) continue;
        accb += g;
        for (int c = 0; c < nci; c++) {
            const float* xc = x + ((size_t)n * cin + ci0 + c) * hin * hin;
#pragma unroll
            for (int ky = 0; ky < 3; ky++)
#pragma unroll
                for (int kx = 0; kx < 3; kx++) {
                    const int iy = oy * stride + ky - 1, ix = ox * stride + kx - 1;
                    if (iy >= 0 && iy < hin && ix >= 0 && ix < hin)
                        acc[c][ky * 3 + kx] = fmaf(g, xc[iy * hin + ix], acc[c][ky * 3 + kx]);
                }
        }
    }
    // block reduction: warp sums, then the 8 warps' sums in order
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 8; c++)
#pragma unroll
        for (int k = 0; k < 9; k++) {
            float v = acc[c][k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[c * 9 + k][wid] = v;
        }
    for (int o = 16; o > 0; o >>= 1) accb += __shfl_xor_sync(0xffffffffu, accb, o);
    if (lane == 0) red[72][wid] = accb;
    __syncthreads();
    if (threadIdx.x < 73) {
        float s = 0.f;
        for (int w = 0; w < 8; w++) s += red[threadIdx.x][w];
        if (threadIdx.x == 72) {
            if (blockIdx.y == 0) atomicAdd(db + co, s);
        } else {
            const int c = threadIdx.x / 9, k = threadIdx.x % 9;
            if (c < nci) atomicAdd(dW + ((size_t)co * cin + ci0 + c) * 9 + k, s);
        }
    }
}

// ------------------------------------------------------------ dense ---
// C[m][n] (+)= sum_k A(m, k) B(k, n); A(m, k) = A[m lda + k] or A[k lda + m]
// (transA), B(k, n) = B[k ldb + n] or B[n ldb + k] (transB).  Optional bias
// per column, ReLU, bf16 rounding of B (weights).  16 x 16 tiles.
__global__ void k_dense(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C,
                        int M, int N, int K, int lda, int ldb, int ldc, int transA, int transB,
                        const float* __restrict__ bias, int relu, int accumulate, int bfB)
{
    __shared__ float As[16][17], Bs[16][17];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int m = blockIdx.y * 16 + ty, n = blockIdx.x * 16 + tx;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        {
            const int mm = blockIdx.y * 16 + ty, kk = k0 + tx;
            float v = 0.f;
            if (mm < M && kk < K) v = transA ? A[(size_t)kk * lda + mm] : A[(size_t)mm * lda + kk];
            As[ty][tx] = v;
        }
        {
            const int kk = k0 + ty, nn = blockIdx.x * 16 + tx;
            float v = 0.f;
            if (kk < K && nn < N) v = transB ? B[(size_t)nn * ldb + kk] : B[(size_t)kk * ldb + nn];
            Bs[ty][tx] = bf(v, bfB);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; k++) acc = fmaf(As[ty][k], Bs[k][tx], acc);
        __syncthreads();
    }
    if (m < M && n < N) {
        float* c = C + (size_t)m * ldc + n;
        float v = acc + (bias ? bias[n] : 0.f);
        if (relu) v = fmaxf(v, 0.f);
        *c = accumulate ? *c + v : v;
    }
}

// g *= (y > 0): the gradient through a ReLU whose output is y
__global__ void k_relu_bwd(float* __restrict__ g, const float* __restrict__ y, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        if (!(y[i] > 0.f)) g[i] = 0.f;
}

// db[n] += sum_m g[m][n]
__global__ void k_col_sum(const float* __restrict__ g, float* __restrict__ db, int M, int N)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.f;
    for (int m = 0; m < M; m++) s += g[(size_t)m * N + n];
    db[n] += s;
}

// --------------------------------------------------------------- head ---
struct V3 {
    double x, y, z;
};
__device__ inline V3 v3(double a, double b, double c) { return {a, b, c}; }
__device__ inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ inline V3 mul(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ inline V3 cross(V3 a, V3 b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// One thread per image: loss and its gradient with respect to the 68 outputs.
// Rstar: the true rotation, columns r1, r2, r3 (row-major 3x3); tstar: shift.
__global__ void k_head_loss(const float* __restrict__ out, const double* __restrict__ Rstar,
                            const double* __restrict__ tstar, float* __restrict__ gout,
                            double* __restrict__ loss, int N, float scale)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const float* o = out + (size_t)n * kOut;
    const double* Rs = Rstar + (size_t)n * 9;
    const V3 r1 = v3(Rs[0], Rs[3], Rs[6]), r2 = v3(Rs[1], Rs[4], Rs[7]), r3 = v3(Rs[2], Rs[5], Rs[8]);
    double lp[kComp], c[kComp], kap[kComp], maxlp = -1e300;
    V3 b1s[kComp], b2s[kComp], a2s[kComp];
    double n1s[kComp], n2s[kComp];
    // log-softmax of the logits
    double lmax = -1e300;
    for (int k = 0; k < kComp; k++) lmax = fmax(lmax, (double)o[k * 8 + 7]);
    double lsum = 0;
    for (int k = 0; k < kComp; k++) lsum += exp((double)o[k * 8 + 7] - lmax);
    const double llse = lmax + log(lsum);
    for (int k = 0; k < kComp; k++) {
        const float* q = o + k * 8;
        const V3 a1 = v3(q[0], q[1], q[2]), a2 = v3(q[3], q[4], q[5]);
        const double n1 = sqrt(dot(a1, a1)) + 1e-12;
        const V3 b1 = mul(a1, 1.0 / n1);
        const V3 u2 = sub(a2, mul(b1, dot(b1, a2)));
        const double n2 = sqrt(dot(u2, u2)) + 1e-12;
        const V3 b2 = mul(u2, 1.0 / n2);
        const V3 b3 = cross(b1, b2);
        c[k] = 0.5 * (dot(b1, r1) + dot(b2, r2) + dot(b3, r3) - 1.0);
        const double raw = q[6];
        kap[k] = (raw > 20 ? raw : log1p(exp(raw))) + 1e-3;
        lp[k] = (double)q[7] - llse + 1.5 * log(kap[k]) + kap[k] * (c[k] - 1.0);
        maxlp = fmax(maxlp, lp[k]);
        b1s[k] = b1;
        b2s[k] = b2;
        a2s[k] = a2;
        n1s[k] = n1;
        n2s[k] = n2;
    }
    double s = 0;
    for (int k = 0; k < kComp; k++) s += exp(lp[k] - maxlp);
    const double lse = maxlp + log(s);
    double L = -lse;
    float* g = gout + (size_t)n * kOut;
    // responsibilities
    double resp[kComp];
    for (int k = 0; k < kComp; k++) resp[k] = exp(lp[k] - lse);
    for (int k = 0; k < kComp; k++) {
        const float* q = o + k * 8;
        // d(-lse)/d lp_k = -resp_k; d lp_k / d logit_j = delta_kj - softmax_j
        // summed: dL/dlogit_j = -resp_j + softmax_j
        const double sm = exp((double)q[7] - llse);
        g[k * 8 + 7] = (float)(scale * (sm - resp[k]));
        // kappa: d lp / d kappa = 1.5 / kappa + (c - 1); d kappa / d raw = sigmoid(raw)
        const double raw = q[6];
        const double sig = raw > 20 ? 1.0 : 1.0 / (1.0 + exp(-raw));
        g[k * 8 + 6] = (float)(scale * (-resp[k]) * (1.5 / kap[k] + c[k] - 1.0) * sig);
        // rotation: d lp / d c = kappa; dc/db1 = (r1 + b2 x r3) / 2, dc/db2 = (r2 + r3 x b1) / 2
        const double w = -resp[k] * kap[k] * scale;
        const V3 b1 = b1s[k], b2 = b2s[k], a2 = a2s[k];
        V3 gb1 = mul(add(r1, cross(b2, r3)), 0.5 * w);
        const V3 gb2 = mul(add(r2, cross(r3, b1)), 0.5 * w);
        // b2 = u2 / |u2|
        const V3 gu2 = mul(sub(gb2, mul(b2, dot(b2, gb2))), 1.0 / n2s[k]);
        // u2 = a2 - (b1 . a2) b1
        const V3 ga2 = sub(gu2, mul(b1, dot(b1, gu2)));
        gb1 = sub(gb1, add(mul(gu2, dot(b1, a2)), mul(a2, dot(b1, gu2))));
        // b1 = a1 / |a1|
        const V3 ga1 = mul(sub(gb1, mul(b1, dot(b1, gb1))), 1.0 / n1s[k]);
        g[k * 8 + 0] = (float)ga1.x;
        g[k * 8 + 1] = (float)ga1.y;
        g[k * 8 + 2] = (float)ga1.z;
        g[k * 8 + 3] = (float)ga2.x;
        g[k * 8 + 4] = (float)ga2.y;
        g[k * 8 + 5] = (float)ga2.z;
    }
    // shift: 0.5 sum ((t - mu)^2 exp(-lv) + lv)
    for (int d = 0; d < 2; d++) {
        const double mu = o[64 + d], lv = o[66 + d];
        const double diff = tstar[(size_t)n * 2 + d] - mu;
        const double e = exp(-lv);
        L += 0.5 * (diff * diff * e + lv);
        g[64 + d] = (float)(scale * (-diff * e));
        g[66 + d] = (float)(scale * 0.5 * (1.0 - diff * diff * e));
    }
    loss[n] = L;
}

// ------------------------------------------------------------- proposals ---
__device__ inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform in (0, 1) from a counter
__device__ inline double u01(uint64_t seed, uint64_t a, uint64_t b)
{
    const uint64_t z = mix64(seed ^ mix64(a * 0x9E3779B97F4A7C15ull + b));
    return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
__device__ inline double normal(uint64_t seed, uint64_t a, uint64_t b)
{
    const double u1 = u01(seed, a, 2 * b), u2 = u01(seed, a, 2 * b + 1);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// nTrans translations ~ N(mu, exp(lv)) from outputs 64..67, the first one
// the mean (counter-based draws, the same for every proposal kernel).
__device__ void propose_trans(const float* o, int l, int nTrans, uint64_t seed,
                              double* __restrict__ trans)
{
    for (int j = threadIdx.x; j < nTrans; j += blockDim.x)
        for (int d = 0; d < 2; d++) {
            const double mu = o[64 + d], sd = exp(0.5 * (double)o[66 + d]);
            trans[((size_t)l * nTrans + j) * 2 + d] =
                j == 0 ? mu : mu + sd * normal(seed, (uint64_t)l * 1024 + 512 + j, d);
        }
}

// One CTA per particle: decode its 8 components, draw nRot rotations
// (the 8 centres, then components by the mixture weights, each turned by a
// rotation vector ~ N(0, I / kappa)) as quaternions (w >= 0), and nTrans
// translations ~ N(mu, exp(lv)) (the first one the mean).
__global__ void k_propose(const float* __restrict__ out, int nRot, int nTrans, uint64_t seed,
                          double* __restrict__ quat, double* __restrict__ trans)
{
    __shared__ double Rk[kComp][9];
    __shared__ double kap[kComp];
    __shared__ double cdf[kComp];
    const int l = blockIdx.x;
    const float* o = out + (size_t)l * kOut;
    if (threadIdx.x < kComp) {
        const int k = threadIdx.x;
        const float* q = o + k * 8;
        const V3 a1 = v3(q[0], q[1], q[2]), a2 = v3(q[3], q[4], q[5]);
        const V3 b1 = mul(a1, 1.0 / (sqrt(dot(a1, a1)) + 1e-12));
        const V3 u2 = sub(a2, mul(b1, dot(b1, a2)));
        const V3 b2 = mul(u2, 1.0 / (sqrt(dot(u2, u2)) + 1e-12));
        const V3 b3 = cross(b1, b2);
        // columns b1 b2 b3, row-major
        const double m[9] = {b1.x, b2.x, b3.x, b1.y, b2.y, b3.y, b1.z, b2.z, b3.z};
        for (int i = 0; i < 9; i++) Rk[k][i] = m[i];
        const double raw = q[6];
        kap[k] = (raw > 20 ? raw : log1p(exp(raw))) + 1e-3;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = -1e300;
        for (int k = 0; k < kComp; k++) mx = fmax(mx, (double)o[k * 8 + 7]);
        double acc = 0;
        for (int k = 0; k < kComp; k++) {
            acc += exp((double)o[k * 8 + 7] - mx);
            cdf[k] = acc;
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nRot; j += blockDim.x) {
        int k = j;
        double v[3] = {0, 0, 0};
        if (j >= kComp) {
            const double u = u01(seed, (uint64_t)l * 1024 + j, 7) * cdf[kComp - 1];
            k = 0;
            while (k < kComp - 1 && u > cdf[k]) k++;
            const double s = 1.0 / sqrt(kap[k]);
            for (int d = 0; d < 3; d++) v[d] = s * normal(seed, (uint64_t)l * 1024 + j, d);
        }
        // R = R_k exp([v]x) (Rodrigues)
        const double th = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        double E[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        if (th > 0) {
            const double kx = v[0] / th, ky = v[1] / th, kz = v[2] / th;
            const double sn = sin(th), cs = 1 - cos(th);
            const double K[9] = {0, -kz, ky, kz, 0, -kx, -ky, kx, 0};
            double K2[9];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    double t = 0;
                    for (int c = 0; c < 3; c++) t += K[a * 3 + c] * K[c * 3 + b];
                    K2[a * 3 + b] = t;
                }
            for (int i = 0; i < 9; i++) E[i] += sn * K[i] + cs * K2[i];
        }
        double M[9];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double t = 0;
                for (int c = 0; c < 3; c++) t += Rk[k][a * 3 + c] * E[c * 3 + b];
                M[a * 3 + b] = t;
            }
        // matrix -> quaternion (w, x, y, z), w >= 0
        const double tr = M[0] + M[4] + M[8];
        double w = sqrt(fmax(0.0, 1 + tr)) / 2, x = sqrt(fmax(0.0, 1 + M[0] - M[4] - M[8])) / 2,
               y = sqrt(fmax(0.0, 1 - M[0] + M[4] - M[8])) / 2,
               z = sqrt(fmax(0.0, 1 - M[0] - M[4] + M[8])) / 2;
        x = copysign(x, M[7] - M[5]);
        y = copysign(y, M[2] - M[6]);
        z = copysign(z, M[3] - M[1]);
        const double nq = sqrt(w * w + x * x + y * y + z * z);
        double* qo = quat + ((size_t)l * nRot + j) * 4;
        qo[0] = w / nq;
        qo[1] = x / nq;
        qo[2] = y / nq;
        qo[3] = z / nq;
    }
    propose_trans(o, l, nTrans, seed, trans);
}

// ------------------------------------------------------------------------
// Matching mode: outputs 0..63 are an embedding, compared by cosine with
// the embeddings of reference projections of the particle's map.
constexpr int kEmb = 64;

// z = u / sqrt(|u|^2 + 1e-12) for u = out[row][0..63]; inv[row] = the factor.
__global__ void k_emb_norm(const float* __restrict__ out, int n, float* __restrict__ z,
                           float* __restrict__ inv)
{
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    const float* u = out + (size_t)row * kOut;
    const float a = u[lane], b = u[lane + 32];
    float s = a * a + b * b;
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float f = 1.0f / sqrtf(s + 1e-12f);
    z[(size_t)row * kEmb + lane] = a * f;
    z[(size_t)row * kEmb + lane + 32] = b * f;
    if (lane == 0 && inv) inv[row] = f;
}

// S[i][j] = zp[i] . zr[j] / tau
__global__ void k_emb_sim(const float* __restrict__ zp, const float* __restrict__ zr, int n,
                          float invTau, float* __restrict__ S)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= n) return;
    const float* a = zp + (size_t)i * kEmb;
    const float* b = zr + (size_t)j * kEmb;
    float acc = 0.f;
#pragma unroll 16
    for (int d = 0; d < kEmb; d++) acc = fmaf(a[d], b[d], acc);
    S[(size_t)i * n + j] = acc * invTau;
}

// log-sum-exp of every row (blockIdx.y = 0) and column (1) of S
__global__ void k_emb_lse(const float* __restrict__ S, int n, float* __restrict__ rowL,
                          float* __restrict__ colL)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool rows = blockIdx.y == 0;
    const size_t st = rows ? 1 : (size_t)n, base = rows ? (size_t)i * n : (size_t)i;
    float m = -INFINITY;
    for (int k = 0; k < n; k++) m = fmaxf(m, S[base + k * st]);
    double acc = 0.0;
    for (int k = 0; k < n; k++) acc += exp((double)(S[base + k * st] - m));
    (rows ? rowL : colL)[i] = m + (float)log(acc);
}

// G = dL/dS for L = (1/n) sum_i 0.5 (rowL_i - S_ii) + 0.5 (colL_i - S_ii)
__global__ void k_emb_dS(const float* __restrict__ S, const float* __restrict__ rowL,
                         const float* __restrict__ colL, int n, float* __restrict__ G)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= n) return;
    const float sij = S[(size_t)i * n + j];
    const float d = i == j ? 1.f : 0.f;
    G[(size_t)i * n + j] = (0.5f / n) * ((expf(sij - rowL[i]) - d) + (expf(sij - colL[j]) - d));
}

// dOut rows: blockIdx.y = 0 particles (embedding part from G zr, shift part
// from the Gaussian shift loss), 1 references (embedding part from G^T zp,
// zero shift part).  One CTA of 64 threads per row.
__global__ void k_emb_grad(const float* __restrict__ G, const float* __restrict__ zp,
                           const float* __restrict__ zr, const float* __restrict__ invP,
                           const float* __restrict__ invR, const float* __restrict__ outP,
                           const double* __restrict__ tstar, int n, float invTau,
                           const float* __restrict__ S, const float* __restrict__ rowL,
                           const float* __restrict__ colL, float* __restrict__ dP,
                           float* __restrict__ dR, double* __restrict__ loss)
{
    __shared__ float red[2];
    const int i = blockIdx.x, d = threadIdx.x;
    const bool part = blockIdx.y == 0;
    const float* zo = part ? zr : zp;            // the other side
    const float* zs = part ? zp : zr;            // this side
    float acc = 0.f;
    for (int k = 0; k < n; k++) {
        const float g = part ? G[(size_t)i * n + k] : G[(size_t)k * n + i];
        acc = fmaf(g, zo[(size_t)k * kEmb + d], acc);
    }
    const float dz = acc * invTau;
    const float zi = zs[(size_t)i * kEmb + d];
    float c = zi * dz;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((d & 31) == 0) red[d >> 5] = c;
    __syncthreads();
    const float zdz = red[0] + red[1];
    const float f = part ? invP[i] : invR[i];
    float* dOut = (part ? dP : dR) + (size_t)i * kOut;
    dOut[d] = f * (dz - zi * zdz);
    if (d < 4) {
        if (!part) {
            dOut[kEmb + d] = 0.f;
        } else if (d < 2) {
            const float* o = outP + (size_t)i * kOut;
            const double mu = o[64 + d], lv = o[66 + d];
            const double diff = tstar[2 * (size_t)i + d] - mu, e = exp(-lv);
            dOut[64 + d] = (float)(-diff * e / n);
            dOut[66 + d] = (float)(0.5 * (1.0 - diff * diff * e) / n);
        }
    }
    if (part && d == 0) {
        const float* o = outP + (size_t)i * kOut;
        double sh = 0.0;
        for (int k = 0; k < 2; k++) {
            const double mu = o[64 + k], lv = o[66 + k];
            const double diff = tstar[2 * (size_t)i + k] - mu;
            sh += 0.5 * (diff * diff * exp(-lv) + lv);
        }
        const double sii = S[(size_t)i * n + i];
        loss[i] = 0.5 * ((double)rowL[i] - sii) + 0.5 * ((double)colL[i] - sii) + sh;
    }
}

// Inclusive scan of v over the CTA's 256 threads (eight warps); ws: 8 words.
__device__ __forceinline__ unsigned block_scan256(unsigned v, unsigned* ws, unsigned* total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    unsigned before = 0, all = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        before += k < w ? ws[k] : 0u;
        all += ws[k];
    }
    __syncthreads();
    *total = all;
    return before + v;
}

// One CTA (256 threads) per particle: cosine scores of its embedding
// against nRef normalised reference embeddings, and the nRot best
// references (descending score, ties to the lower index) as the rotation
// proposals.  The nRot-th largest score key is found by four 8-bit radix
// passes over order-preserving keys in shared memory; the keys above it and
// the lowest-index keys equal to it are compacted in index order, then
// sorted (bitonic, nSort = nRot rounded up to a power of two).
//
// With table != null, particle l matches the references of its class:
// table[cls[l]] (embeddings, rotations, count) replaces ref / refQuat /
// nRef.  A class without nRot references gets index -1 proposals, which
// the rescoring gather reports as out of range.
__global__ void __launch_bounds__(256)
k_match_propose(const float* __restrict__ out, const float* __restrict__ ref, int nRef,
                int nSort, const double* __restrict__ refQuat, int nRot, int nTrans,
                uint64_t seed, double* __restrict__ quat, double* __restrict__ trans,
                int* __restrict__ idxOut, const RefView* __restrict__ table,
                const int* __restrict__ cls)
{
    extern __shared__ unsigned long long smx[];
    unsigned long long* sel = smx;                                   // [nSort]
    uint32_t* skey = reinterpret_cast<uint32_t*>(smx + nSort);       // [nRef]
    __shared__ float zp[kEmb];
    __shared__ float red[8];
    __shared__ unsigned hist[256];
    __shared__ unsigned ws[8];
    __shared__ unsigned sPrefix, sMask, sK;
    const int l = blockIdx.x, tid = threadIdx.x;
    const float* o = out + (size_t)l * kOut;
    if (table) {
        const int k = cls[l];
        const RefView v = (k >= 0 && k < kMaxClasses) ? table[k] : RefView{nullptr, nullptr, 0};
        if (!v.emb || !v.quat || v.n < nRot) {
            for (int j = tid; j < nRot; j += blockDim.x) {
                if (idxOut) idxOut[(size_t)l * nRot + j] = -1;
                double* qo = quat + ((size_t)l * nRot + j) * 4;
                qo[0] = 1.0;
                qo[1] = qo[2] = qo[3] = 0.0;
            }
            propose_trans(o, l, nTrans, seed, trans);
            return;
        }
        ref = v.emb;
        refQuat = v.quat;
        nRef = v.n;
    }
    if (tid < kEmb) {
        const float a = o[tid];
        float q = a * a;
        for (int k = 16; k; k >>= 1) q += __shfl_xor_sync(0xffffffffu, q, k);
        if ((tid & 31) == 0) red[tid >> 5] = q;
    }
    __syncthreads();
    if (tid < kEmb) zp[tid] = o[tid] / sqrtf(red[0] + red[1] + 1e-12f);
    if (tid == 0) {
        sPrefix = 0u;
        sMask = 0u;
        sK = (unsigned)nRot;
    }
    __syncthreads();
    for (int j = tid; j < nRef; j += blockDim.x) {
        const float4* r = reinterpret_cast<const float4*>(ref + (size_t)j * kEmb);
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < kEmb / 4; q++) {
            const float4 v = __ldg(r + q);
            acc = fmaf(zp[4 * q], v.x, acc);
            acc = fmaf(zp[4 * q + 1], v.y, acc);
            acc = fmaf(zp[4 * q + 2], v.z, acc);
            acc = fmaf(zp[4 * q + 3], v.w, acc);
        }
        const unsigned b = __float_as_uint(acc);
        skey[j] = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    }
    // the nRot-th largest key
    for (int shift = 24; shift >= 0; shift -= 8) {
        hist[tid] = 0u;
        __syncthreads();
        const unsigned prefix = sPrefix, mask = sMask;
        for (int j = tid; j < nRef; j += blockDim.x) {
            const unsigned k = skey[j];
            if ((k & mask) == prefix) atomicAdd(&hist[(k >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (tid == 0) {
            unsigned kth = sK, acc = 0u;
            int d = 255;
            for (; d > 0; d--) {
                if (acc + hist[d] >= kth) break;
                acc += hist[d];
            }
            sK = kth - acc;
            sPrefix = prefix | ((unsigned)d << shift);
            sMask = mask | (255u << shift);
        }
        __syncthreads();
    }
    const unsigned T = sPrefix, kEq = sK;
    // compaction in index order: thread t holds indices [t per, (t + 1) per)
    const int per = (nRef + blockDim.x - 1) / blockDim.x;
    const int j0 = min(nRef, tid * per), j1 = min(nRef, j0 + per);
    unsigned cg = 0u, ce = 0u;
    for (int j = j0; j < j1; j++) {
        cg += skey[j] > T;
        ce += skey[j] == T;
    }
    unsigned totG, totE;
    unsigned pg = block_scan256(cg, ws, &totG) - cg;
    unsigned pe = block_scan256(ce, ws, &totE) - ce;
    for (int j = j0; j < j1; j++) {
        const unsigned k = skey[j];
        const unsigned long long key = ((unsigned long long)k << 32) | (0xFFFFFFFFu - (unsigned)j);
        if (k > T) {
            sel[pg++] = key;
        } else if (k == T) {
            if (pe < kEq) sel[totG + pe] = key;
            pe++;
        }
    }
    for (int j = nRot + tid; j < nSort; j += blockDim.x) sel[j] = 0ull;
    __syncthreads();
    for (int size = 2; size <= nSort; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = tid; t < nSort / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool desc = (lo & size) == 0;
                const unsigned long long a = sel[lo], b = sel[hi];
                if ((a < b) == desc) {
                    sel[lo] = b;
                    sel[hi] = a;
                }
            }
            __syncthreads();
        }
    for (int j = tid; j < nRot; j += blockDim.x) {
        const int idx = (int)(0xFFFFFFFFu - (unsigned int)(sel[j] & 0xFFFFFFFFu));
        if (idxOut) idxOut[(size_t)l * nRot + j] = idx;
        const double* src = refQuat + 4 * (size_t)idx;
        double* qo = quat + ((size_t)l * nRot + j) * 4;
        for (int c = 0; c < 4; c++) qo[c] = src[c];
    }
    propose_trans(o, l, nTrans, seed, trans);
}

__global__ void k_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, size_t n, float lr, float b1, float b2, float c1,
                       float c2, float eps)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

}  // namespace
}  // namespace tg3

using namespace tg3;

struct tg3_cnn {
    int device = 0;
    cudaStream_t stream = nullptr;
    size_t nParams = 0;
    size_t off[kLayers][2];     // weight / bias offsets in the parameter vector
    float* params = nullptr;    // FP32 master weights and biases
    float* grads = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    long long step = 0;
    int roundW = 1;             // weights used in bf16 (0: FP32, for gradient checks)
    int cap = 0;                // images the activation buffers hold
    float* act[kLayers + 1] = {};   // act[0] input copy .. act[8] outputs
    float* gact[kLayers + 1] = {};
    double* Rstar = nullptr;
    double* loss = nullptr;
    // tensor-core inference: repacked bf16 weights, bf16 NHWC activations
    __nv_bfloat16* tcW = nullptr;
    size_t tcOff[kLayers] = {};
    int tcCap = 0;
    __nv_bfloat16* tcAct[kLayers] = {};     // outputs of layers 0 .. 6
    int* tcFlag = nullptr;
    float* tcPartial = nullptr;             // split-K sums of the dense layer
    // contrastive scratch (matching mode), grown as needed
    int embCap = 0;
    float* emb = nullptr;       // zp, zr [n][64]; invP, invR [n]; rowL, colL [n]; S, G [n][n]
    double* embLoss = nullptr;
};

namespace {

size_t act_size(int l)
{
    if (l == 0) return 64 * 64;
    const LayerShape& s = kShape[l - 1];
    return s.stride ? (size_t)s.cout * s.hout * s.hout : (size_t)s.cout;
}

int ensure_capacity(tg3_cnn* net, int n)
{
    if (n <= net->cap) return TG3_OK;
    TG3_CUDA(cudaStreamSynchronize(net->stream));
    for (int l = 0; l <= kLayers; l++) {
        cudaFree(net->act[l]);
        cudaFree(net->gact[l]);
        net->act[l] = net->gact[l] = nullptr;
    }
    cudaFree(net->Rstar);
    cudaFree(net->loss);
    for (int l = 0; l <= kLayers; l++) {
        TG3_CUDA(cudaMalloc(&net->act[l], sizeof(float) * act_size(l) * n));
        TG3_CUDA(cudaMalloc(&net->gact[l], sizeof(float) * act_size(l) * n));
    }
    TG3_CUDA(cudaMalloc(&net->Rstar, sizeof(double) * 9 * n));
    TG3_CUDA(cudaMalloc(&net->loss, sizeof(double) * n));
    net->cap = n;
    return TG3_OK;
}

int forward(tg3_cnn* net, int n)
{
    cudaStream_t s = net->stream;
    for (int l = 0; l < kLayers; l++) {
        const LayerShape& sh = kShape[l];
        const float* W = net->params + net->off[l][0];
        const float* b = net->params + net->off[l][1];
        if (sh.stride) {
            dim3 grid((sh.hout * sh.hout + 255) / 256, (sh.cout + 15) / 16, n);
            k_conv_fwd<<<grid, 256, 0, s>>>(net->act[l], W, b, net->act[l + 1], sh.cin, sh.cout,
                                             sh.hin, sh.hout, sh.stride, 1, net->roundW);
        } else {
            dim3 grid((sh.cout + 15) / 16, (n + 15) / 16);
            k_dense<<<grid, dim3(16, 16), 0, s>>>(net->act[l], W, net->act[l + 1], n, sh.cout,
                                                  sh.cin, sh.cin, sh.cin, sh.cout, 0, 1, b,
                                                  l < kLayers - 1, 0, net->roundW);
        }
        TG3_LAUNCH_CHECK("network forward");
    }
    return TG3_OK;
}

// gact[kLayers] holds dL/d outputs; fills grads (accumulating)
int backward(tg3_cnn* net, int n)
{
    cudaStream_t s = net->stream;
    for (int l = kLayers - 1; l >= 0; l--) {
        const LayerShape& sh = kShape[l];
        const float* W = net->params + net->off[l][0];
        float* dW = net->grads + net->off[l][0];
        float* db = net->grads + net->off[l][1];
        float* gy = net->gact[l + 1];
        // through this layer's ReLU (all but the last)
        if (l < kLayers - 1) {
            const size_t cnt = act_size(l + 1) * n;
            k_relu_bwd<<<cnn_grid(cnt, 256), 256, 0, s>>>(gy, net->act[l + 1], cnt);
        }
        if (sh.stride) {
            const int imgPerCta = 8;
            dim3 gw(sh.cout, (sh.cin + 7) / 8, (n + imgPerCta - 1) / imgPerCta);
            k_conv_bwd_weight<<<gw, 256, 0, s>>>(net->act[l], gy, dW, db, n, sh.cin, sh.cout,
                                                  sh.hin, sh.hout, sh.stride, imgPerCta);
            if (l > 0) {
                dim3 gd((sh.hin * sh.hin + 255) / 256, (sh.cin + 15) / 16, n);
                k_conv_bwd_data<<<gd, 256, 0, s>>>(gy, W, net->gact[l], sh.cin, sh.cout, sh.hin,
                                                    sh.hout, sh.stride, net->roundW);
            }
        } else {
            // dW[o][i] += sum_n gy[n][o] x[n][i]; db[o] += sum_n gy[n][o]; dx = gy W
            dim3 g1((sh.cin + 15) / 16, (sh.cout + 15) / 16);
            k_dense<<<g1, dim3(16, 16), 0, s>>>(gy, net->act[l], dW, sh.cout, sh.cin, n, sh.cout,
                                                sh.cin, sh.cin, 1, 0, nullptr, 0, 1, 0);
            k_col_sum<<<(sh.cout + 255) / 256, 256, 0, s>>>(gy, db, n, sh.cout);
            dim3 g2((sh.cin + 15) / 16, (n + 15) / 16);
            k_dense<<<g2, dim3(16, 16), 0, s>>>(gy, W, net->gact[l], n, sh.cin, sh.cout, sh.cout,
                                                sh.cin, sh.cin, 0, 0, nullptr, 0, 0, net->roundW);
        }
        TG3_LAUNCH_CHECK("network backward");
    }
    return TG3_OK;
}

// He-normal weights from a counter-based generator (splitmix64 + Box-Muller),
// zero biases.
void init_params(std::vector<float>& h, const tg3_cnn* net, uint64_t seed)
{
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
    for (int l = 0; l < kLayers; l++) {
        const LayerShape& s = kShape[l];
        const size_t nw = weight_count(s);
        const double fan = s.stride ? s.cin * 9.0 : (double)s.cin;
        const double sd = sqrt(2.0 / fan) * (l == kLayers - 1 ? 0.1 : 1.0);
        for (size_t i = 0; i < nw; i++) {
            const double u1 = unif(), u2 = unif();
            h[net->off[l][0] + i] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
    }
}

}  // namespace

extern "C" int tg3_cnn_create(tg3_cnn** out, int device, unsigned long long seed)
{
    if (!out) return fail(TG3_ERR_ARG, "null output");
    TG3_CUDA(cudaSetDevice(device));
    tg3_cnn* net = new tg3_cnn();
    net->device = device;
    size_t o = 0;
    for (int l = 0; l < kLayers; l++) {
        net->off[l][0] = o;
        o += weight_count(kShape[l]);
        net->off[l][1] = o;
        o += kShape[l].cout;
    }
    net->nParams = o;
    if (cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&net->params, sizeof(float) * o) != cudaSuccess ||
        cudaMalloc(&net->grads, sizeof(float) * o) != cudaSuccess ||
        cudaMalloc(&net->m, sizeof(float) * o) != cudaSuccess ||
        cudaMalloc(&net->v, sizeof(float) * o) != cudaSuccess) {
        tg3_cnn_destroy(net);
        return fail(TG3_ERR_ALLOC, "network allocation");
    }
    std::vector<float> h(o, 0.f);
    init_params(h, net, seed);
    cudaMemcpy(net->params, h.data(), sizeof(float) * o, cudaMemcpyHostToDevice);
    cudaMemset(net->grads, 0, sizeof(float) * o);
    cudaMemset(net->m, 0, sizeof(float) * o);
    cudaMemset(net->v, 0, sizeof(float) * o);
    *out = net;
    return TG3_OK;
}

extern "C" int tg3_cnn_destroy(tg3_cnn* net)
{
    if (!net) return TG3_OK;
    cudaSetDevice(net->device);
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (int l = 0; l <= kLayers; l++) {
        cudaFree(net->act[l]);
        cudaFree(net->gact[l]);
    }
    cudaFree(net->Rstar);
    cudaFree(net->loss);
    cudaFree(net->emb);
    cudaFree(net->embLoss);
    cudaFree(net->tcW);
    cudaFree(net->tcFlag);
    cudaFree(net->tcPartial);
    for (int l = 0; l < kLayers; l++) cudaFree(net->tcAct[l]);
    cudaFree(net->params);
    cudaFree(net->grads);
    cudaFree(net->m);
    cudaFree(net->v);
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
    return TG3_OK;
}

extern "C" size_t tg3_cnn_param_count(const tg3_cnn* net) { return net ? net->nParams : 0; }

extern "C" int tg3_cnn_params(tg3_cnn* net, float* host, int set)
{
    if (!net || !host) return fail(TG3_ERR_ARG, "null argument");
    TG3_CUDA(cudaSetDevice(net->device));
    TG3_CUDA(cudaStreamSynchronize(net->stream));
    TG3_CUDA(cudaMemcpy(set ? (void*)net->params : (void*)host, set ? (const void*)host : net->params,
                        sizeof(float) * net->nParams,
                        set ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost));
    return TG3_OK;
}

extern "C" int tg3_cnn_grads(tg3_cnn* net, float* host)
{
    if (!net || !host) return fail(TG3_ERR_ARG, "null argument");
    TG3_CUDA(cudaSetDevice(net->device));
    TG3_CUDA(cudaStreamSynchronize(net->stream));
    TG3_CUDA(cudaMemcpy(host, net->grads, sizeof(float) * net->nParams, cudaMemcpyDeviceToHost));
    return TG3_OK;
}

// outputs [n][68] (device) for images [n][64][64] (device)
extern "C" int tg3_cnn_forward(tg3_cnn* net, const float* img, int n, float* out)
{
    if (!net || !img || !out || n <= 0) return fail(TG3_ERR_ARG, "bad forward arguments");
    TG3_CUDA(cudaSetDevice(net->device));
    int st = ensure_capacity(net, n);
    if (st) return st;
    TG3_CUDA(cudaMemcpyAsync(net->act[0], img, sizeof(float) * 64 * 64 * n,
                             cudaMemcpyDeviceToDevice, net->stream));
    if ((st = forward(net, n))) return st;
    TG3_CUDA(cudaMemcpyAsync(out, net->act[kLayers], sizeof(float) * kOut * n,
                             cudaMemcpyDeviceToDevice, net->stream));
    TG3_CUDA(cudaStreamSynchronize(net->stream));
    return TG3_OK;
}

// Loss of a batch (mean over images, returned on the host) and, with
// `accumulate_grads`, the gradient of that mean added to the network's
// gradient buffer.  Rstar [n][9] row-major true rotations, tstar [n][2].
extern "C" int tg3_cnn_loss(tg3_cnn* net, const float* img, int n, const double* Rstar,
                            const double* tstar, int accumulate_grads, double* lossOut)
{
    if (!net || !img || !Rstar || !tstar || n <= 0) return fail(TG3_ERR_ARG, "bad loss arguments");
    TG3_CUDA(cudaSetDevice(net->device));
    int st = ensure_capacity(net, n);
    if (st) return st;
    cudaStream_t s = net->stream;
    TG3_CUDA(cudaMemcpyAsync(net->act[0], img, sizeof(float) * 64 * 64 * n,
                             cudaMemcpyDeviceToDevice, s));
    if ((st = forward(net, n))) return st;
    k_head_loss<<<(n + 127) / 128, 128, 0, s>>>(net->act[kLayers], Rstar, tstar,
                                                 net->gact[kLayers], net->loss, n, 1.0f / n);
    TG3_LAUNCH_CHECK("network loss");
    if (accumulate_grads && (st = backward(net, n))) return st;
    std::vector<double> h(n);
    TG3_CUDA(cudaMemcpyAsync(h.data(), net->loss, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaStreamSynchronize(s));
    double sum = 0;
    for (double x : h) sum += x;
    if (lossOut) *lossOut = sum / n;
    return TG3_OK;
}

extern "C" int tg3_cnn_zero_grads(tg3_cnn* net)
{
    if (!net) return fail(TG3_ERR_ARG, "null network");
    TG3_CUDA(cudaSetDevice(net->device));
    TG3_CUDA(cudaMemsetAsync(net->grads, 0, sizeof(float) * net->nParams, net->stream));
    return TG3_OK;
}

extern "C" int tg3_cnn_adam(tg3_cnn* net, float lr)
{
    if (!net) return fail(TG3_ERR_ARG, "null network");
    TG3_CUDA(cudaSetDevice(net->device));
    net->step++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)net->step), c2 = 1.f - powf(b2, (float)net->step);
    k_adam<<<cnn_grid(net->nParams, 256), 256, 0, net->stream>>>(net->params, net->grads, net->m,
                                                                  net->v, net->nParams, lr, b1, b2,
                                                                  c1, c2, 1e-8f);
    TG3_LAUNCH_CHECK("adam");
    return TG3_OK;
}

extern "C" int tg3_cnn_set_bf16(tg3_cnn* net, int enable)
{
    if (!net) return fail(TG3_ERR_ARG, "null network");
    net->roundW = enable != 0;
    return TG3_OK;
}

extern "C" int tg3_cnn_propose(const float* out, int n, int nRot, int nTrans,
                               unsigned long long seed, double* quat, double* trans, void* stream)
{
    if (!out || !quat || !trans || n <= 0 || nRot < kComp || nRot > 512 || nTrans <= 0 ||
        nTrans > 512)
        return fail(TG3_ERR_ARG, "bad proposal arguments (8 <= nRot <= 512, nTrans <= 512)");
    k_propose<<<n, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, nRot, nTrans, seed, quat,
                                                                 trans);
    TG3_LAUNCH_CHECK("proposals");
    return TG3_OK;
}

// Add to the gradient buffer the gradient of a loss whose derivative with
// respect to the outputs for images img [n][64][64] is dOut [n][68]
// (device; the forward pass is run again to rebuild the activations).
extern "C" int tg3_cnn_backward(tg3_cnn* net, const float* img, int n, const float* dOut)
{
    if (!net || !img || !dOut || n <= 0) return fail(TG3_ERR_ARG, "bad backward arguments");
    TG3_CUDA(cudaSetDevice(net->device));
    int st = ensure_capacity(net, n);
    if (st) return st;
    cudaStream_t s = net->stream;
    TG3_CUDA(cudaMemcpyAsync(net->act[0], img, sizeof(float) * 64 * 64 * n,
                             cudaMemcpyDeviceToDevice, s));
    if ((st = forward(net, n))) return st;
    TG3_CUDA(cudaMemcpyAsync(net->gact[kLayers], dOut, sizeof(float) * kOut * n,
                             cudaMemcpyDeviceToDevice, s));
    return backward(net, n);
}

// Matching loss of a batch of n particles and their n reference
// projections (outputs outP, outR [n][68], device): symmetric InfoNCE on the
// cosine similarities / tau of the normalised embeddings (outputs 0..63),
// particle i's positive being reference i, plus the Gaussian shift loss of
// the particles' outputs 64..67 against tstar [n][2].  Writes dL/d outputs
// (dOutP, dOutR) and the mean loss (host).  n <= 1024.
extern "C" int tg3_cnn_contrastive(tg3_cnn* net, const float* outP, const float* outR, int n,
                                   const double* tstar, float tau, float* dOutP, float* dOutR,
                                   double* lossOut)
{
    if (!net || !outP || !outR || !tstar || !dOutP || !dOutR || n <= 1 || n > 1024 ||
        !(tau > 0.f))
        return fail(TG3_ERR_ARG, "bad contrastive arguments (1 < n <= 1024, tau > 0)");
    TG3_CUDA(cudaSetDevice(net->device));
    cudaStream_t s = net->stream;
    if (n > net->embCap) {
        TG3_CUDA(cudaStreamSynchronize(s));
        cudaFree(net->emb);
        cudaFree(net->embLoss);
        net->emb = nullptr;
        net->embLoss = nullptr;
        net->embCap = 0;
        TG3_CUDA(cudaMalloc(&net->emb, sizeof(float) * ((size_t)2 * kEmb * n + 4 * n +
                                                        2 * (size_t)n * n)));
        TG3_CUDA(cudaMalloc(&net->embLoss, sizeof(double) * n));
        net->embCap = n;
    }
    float* zp = net->emb;
    float* zr = zp + (size_t)kEmb * n;
    float* invP = zr + (size_t)kEmb * n;
    float* invR = invP + n;
    float* rowL = invR + n;
    float* colL = rowL + n;
    float* S = colL + n;
    float* G = S + (size_t)n * n;
    const float invTau = 1.0f / tau;
    k_emb_norm<<<(n + 7) / 8, 256, 0, s>>>(outP, n, zp, invP);
    k_emb_norm<<<(n + 7) / 8, 256, 0, s>>>(outR, n, zr, invR);
    k_emb_sim<<<dim3((n + 127) / 128, n), 128, 0, s>>>(zp, zr, n, invTau, S);
    k_emb_lse<<<dim3((n + 127) / 128, 2), 128, 0, s>>>(S, n, rowL, colL);
    k_emb_dS<<<dim3((n + 127) / 128, n), 128, 0, s>>>(S, rowL, colL, n, G);
    k_emb_grad<<<dim3(n, 2), kEmb, 0, s>>>(G, zp, zr, invP, invR, outP, tstar, n, invTau, S, rowL,
                                           colL, dOutP, dOutR, net->embLoss);
    TG3_LAUNCH_CHECK("contrastive loss");
    std::vector<double> h(n);
    TG3_CUDA(cudaMemcpyAsync(h.data(), net->embLoss, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaStreamSynchronize(s));
    double sum = 0;
    for (double x : h) sum += x;
    if (lossOut) *lossOut = sum / n;
    return TG3_OK;
}

// Normalised embeddings z [n][64] of outputs out [n][68] (device).
extern "C" int tg3_cnn_embed(const float* out, int n, float* z, void* stream)
{
    if (!out || !z || n <= 0) return fail(TG3_ERR_ARG, "bad embed arguments");
    k_emb_norm<<<(n + 7) / 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(out, n, z, nullptr);
    TG3_LAUNCH_CHECK("embeddings");
    return TG3_OK;
}

// Rotation proposals by matching: for every particle (outputs out [n][68]),
// the nRot references of highest cosine score (ref [nRef][64] normalised,
// refQuat [nRef][4]) with their indices (idx [n][nRot], may be NULL), and
// nTrans translations from the shift outputs.
extern "C" int tg3_cnn_match_propose(const float* out, int n, const float* ref, int nRef,
                                     const double* refQuat, int nRot, int nTrans,
                                     unsigned long long seed, double* quat, double* trans,
                                     int* idx, void* stream)
{
    if (!out || !ref || !refQuat || !quat || !trans || n <= 0 || nRef <= 0 || nRef > 16384 ||
        nRot <= 0 || nRot > nRef || nTrans <= 0 || nTrans > 512)
        return fail(TG3_ERR_ARG, "bad match arguments (nRot <= nRef <= 16384, nTrans <= 512)");
    int p2 = 1;
    while (p2 < nRot) p2 <<= 1;
    const size_t smem = sizeof(unsigned long long) * p2 + sizeof(uint32_t) * (size_t)nRef;
    if (smem > 200 * 1024) return fail(TG3_ERR_ARG, "match sizes need too much shared memory");
    TG3_CUDA(cudaFuncSetAttribute(k_match_propose, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    k_match_propose<<<n, 256, smem, static_cast<cudaStream_t>(stream)>>>(
        out, ref, nRef, p2, refQuat, nRot, nTrans, seed, quat, trans, idx, nullptr, nullptr);
    TG3_LAUNCH_CHECK("match proposals");
    return TG3_OK;
}

// Every particle against the references of its own class (RefView table).
cudaError_t tg3::launch_match_propose_classes(const float* out, int n, const RefView* table,
                                              const int* cls, int maxRef, int nRot, int nTrans,
                                              unsigned long long seed, double* quat,
                                              double* trans, int* idx, cudaStream_t st)
{
    if (!out || !table || !cls || !quat || !trans || n <= 0 || maxRef <= 0 || maxRef > 16384 ||
        nRot <= 0 || nRot > maxRef || nTrans <= 0 || nTrans > 512)
        return cudaErrorInvalidValue;
    int p2 = 1;
    while (p2 < nRot) p2 <<= 1;
    const size_t smem = sizeof(unsigned long long) * p2 + sizeof(uint32_t) * (size_t)maxRef;
    if (smem > 200 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_match_propose,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_match_propose<<<n, 256, smem, st>>>(out, nullptr, maxRef, p2, nullptr, nRot, nTrans, seed,
                                          quat, trans, idx, table, cls);
    return cudaGetLastError();
}

namespace tg3 {
namespace {

// Rows and K (padded) of every layer's repacked weights for the inference
// path: conv 0 [32][9]; convs 1..5 [cout][9 cin] (tap-major K); dense 6
// [256][8192] with K in NHWC order (y, x, c); dense 7 [68][256].
void tc_dims(int l, int* rows, int* kpad)
{
    const LayerShape& s = kShape[l];
    if (l == 0) {
        *rows = s.cout;
        *kpad = 9;
    } else if (s.stride) {
        *rows = s.cout;
        *kpad = 9 * s.cin;
    } else {
        *rows = s.cout;
        *kpad = s.cin;
    }
}

__global__ void k_tc_repack(const float* __restrict__ W, int l, int rows, int kpad, int cin,
                            int hin, __nv_bfloat16* __restrict__ out)
{
    const size_t total = (size_t)rows * kpad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
         i += (size_t)gridDim.x * blockDim.x) {
        const int o = (int)(i / kpad), k = (int)(i % kpad);
        size_t src;
        if (l == 0) {
            src = (size_t)o * 9 + k;                                  // [o][0][ky][kx]
        } else if (l <= 5) {
            const int tap = k / cin, ci = k % cin;                    // k = tap cin + ci
            src = ((size_t)o * cin + ci) * 9 + tap;
        } else if (l == 6) {
            const int c = k % 128, yx = k / 128;                      // k = (y 8 + x) 128 + c
            src = (size_t)o * kpad + (size_t)c * 64 + yx;
        } else {
            src = (size_t)o * kpad + k;
        }
        out[i] = __float2bfloat16_rn(W[src]);
    }
    (void)hin;
}

constexpr int kInferChunk = 2048;
constexpr int kDenseSplit = 16;

int tc_prepare(tg3_cnn* net, int n)
{
    cudaStream_t s = net->stream;
    if (!net->tcW) {
        size_t o = 0;
        for (int l = 0; l < kLayers; l++) {
            int rows, kpad;
            tc_dims(l, &rows, &kpad);
            net->tcOff[l] = o;
            o += (size_t)rows * kpad;
            o = (o + 63) & ~(size_t)63;
        }
        TG3_CUDA(cudaMalloc(&net->tcW, sizeof(__nv_bfloat16) * o));
        TG3_CUDA(cudaMalloc(&net->tcFlag, sizeof(int)));
        TG3_CUDA(cudaMemset(net->tcFlag, 0, sizeof(int)));
    }
    for (int l = 0; l < kLayers; l++) {
        int rows, kpad;
        tc_dims(l, &rows, &kpad);
        k_tc_repack<<<cnn_grid((size_t)rows * kpad, 256), 256, 0, s>>>(
            net->params + net->off[l][0], l, rows, kpad, kShape[l].cin, kShape[l].hin,
            net->tcW + net->tcOff[l]);
    }
    TG3_LAUNCH_CHECK("weights repack");
    const int cap = std::min(n, kInferChunk);
    if (cap > net->tcCap) {
        TG3_CUDA(cudaStreamSynchronize(s));
        for (int l = 0; l < kLayers; l++) {
            cudaFree(net->tcAct[l]);
            net->tcAct[l] = nullptr;
        }
        net->tcCap = 0;
        cudaFree(net->tcPartial);
        net->tcPartial = nullptr;
        for (int l = 0; l < kLayers - 1; l++)
            TG3_CUDA(cudaMalloc(&net->tcAct[l], sizeof(__nv_bfloat16) * act_size(l + 1) * cap));
        TG3_CUDA(cudaMalloc(&net->tcPartial,
                            sizeof(float) * kDenseSplit * (size_t)cap * kShape[6].cout));
        net->tcCap = cap;
    }
    return TG3_OK;
}

}  // namespace
}  // namespace tg3

// Inference forward with bf16 activations (tensor cores for the wide
// layers): outputs [n][68] (device) for images [n][64][64] (device).
extern "C" int tg3_cnn_infer(tg3_cnn* net, const float* img, int n, float* out)
{
    if (!net || !img || !out || n <= 0) return fail(TG3_ERR_ARG, "bad inference arguments");
    TG3_CUDA(cudaSetDevice(net->device));
    int st = tc_prepare(net, n);
    if (st) return st;
    cudaStream_t s = net->stream;
    for (int i0 = 0; i0 < n; i0 += kInferChunk) {
        const int m = std::min(kInferChunk, n - i0);
        const float* b0 = net->params + net->off[0][1];
        TG3_CUDA(launch_conv1_nhwc(img + (size_t)i0 * 64 * 64, net->tcW + net->tcOff[0], b0, m,
                                   64, net->tcAct[0], s));
        for (int l = 1; l <= 6; l++) {
            const LayerShape& sh = kShape[l];
            int rows, kpad;
            tc_dims(l, &rows, &kpad);
            ConvTcArgs a;
            a.in = net->tcAct[l - 1];
            a.w = net->tcW + net->tcOff[l];
            a.bias = net->params + net->off[l][1];
            a.out = net->tcAct[l];
            a.n = m;
            if (sh.stride) {
                a.H = a.W = sh.hin;
                a.Ho = a.Wo = sh.hout;
                a.Cin = sh.cin;
                a.ks = 3;
                a.stride = sh.stride;
                a.pad = 1;
            } else {
                a.H = a.W = a.Ho = a.Wo = 1;
                a.Cin = sh.cin;
                a.ks = 1;
                a.stride = 1;
                a.pad = 0;
            }
            a.Cout = sh.cout;
            a.coutPad = sh.cout;
            a.Kpad = kpad;
            a.tmemCols = sh.cout < 32 ? 32 : sh.cout;
            a.relu = 1;
            a.flag = net->tcFlag;
            // the dense layer: few rows of 128 images, 256 K blocks -> 16 K slices
            a.kSplit = sh.stride ? 1 : kDenseSplit;
            a.partial = sh.stride ? nullptr : net->tcPartial;
            TG3_CUDA(launch_conv_tc(a, s));
        }
        TG3_CUDA(launch_fc_out(net->tcAct[6], net->tcW + net->tcOff[7],
                               net->params + net->off[7][1], m, kShape[7].cin, kOut,
                               out + (size_t)i0 * kOut, s));
    }
    TG3_CUDA(cudaStreamSynchronize(s));
    int flag = 0;
    TG3_CUDA(cudaMemcpy(&flag, net->tcFlag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        cudaMemset(net->tcFlag, 0, sizeof(int));
        return fail(TG3_ERR_TIMEOUT, "tensor-core wait expired in the network");
    }
    return TG3_OK;
}
