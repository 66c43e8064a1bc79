// tg3_learned.cu -- the learned E-step: the pose network's proposals, scored
// by the exact likelihood, with the global search as the fallback.
//
// In THUNDER the first expectation of a refinement is the global search:
// every particle against every rotation of a uniform grid x a translation
// grid (Optimiser::doGlobalSearch, src/Optimiser.cpp:633-1136; on the GPU
// expectGlobal3D, gpu/interface/Interface.h:221).  The learned E-step seeds
// each particle's hypotheses from the pose network instead:
//   1. the network embeds the particle's 64 x 64 image (tg3_cnn_infer);
//   2. the nRot references of the particle's class whose embeddings match it
//      best, with nTrans shifts drawn from the network's shift output
//      (k_match_propose over the class's RefView);
//   3. every proposed (rotation, translation) is scored by the exact
//      likelihood from the class's projection bank (the bank-row local phase);
//   4. the proposal's confidence, (best - median) / (1.4826 MAD) of its
//      log-likelihoods, is compared with a threshold; a particle below it
//      falls back to the global search over the bank's rotations x the
//      caller's translation grid, with the bank's projections reused;
//   5. each particle's best pose (argmax of its rotation and translation
//      marginals) and its best log-likelihood are returned.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <algorithm>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {

namespace {

constexpr int kEmbDim = 64;
constexpr int kNetOut = 68;
constexpr int kMaxPeakN = 16384;     // hypotheses per particle the confidence kernel sorts

__global__ void k_fill_f64(double* __restrict__ p, size_t n, double v)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = v;
}

// Ascending bitonic sort of n (a power of two) floats in shared memory.
__device__ void bitonic_sort_asc(float* v, int n)
{
    for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = (lo & size) == 0;
                const float a = v[lo], b = v[hi];
                if ((a > b) == asc) {
                    v[lo] = b;
                    v[hi] = a;
                }
            }
            __syncthreads();
        }
}

// Median of the n sorted values v[0 .. n) (the mean of the middle two for
// even n, as numpy's median).
__device__ __forceinline__ double sorted_median(const float* v, int n)
{
    return (n & 1) ? (double)v[n / 2] : 0.5 * ((double)v[n / 2 - 1] + (double)v[n / 2]);
}

// The deviations |v - med| of the sorted values v[0 .. n) (rounded to float)
// form two ascending runs: med - v[s - 1 - j] over the s values below med,
// and v[s + j] - med over the rest.  dev_kth returns the k-th smallest
// (0-based) of their union by a binary search over how many come from the
// left run -- the same value a sort of all n deviations would put at k.
__device__ __forceinline__ float dev_left(const float* v, int s, double med, int j)
{
    return (float)fabs((double)v[s - 1 - j] - med);
}

__device__ __forceinline__ float dev_right(const float* v, int s, double med, int j)
{
    return (float)fabs((double)v[s + j] - med);
}

__device__ float dev_kth(const float* v, int n, int s, double med, int k)
{
    const int a = s, b = n - s;
    int lo = max(0, k + 1 - b), hi = min(k + 1, a);   // values taken from the left run
    while (lo < hi) {
        const int i = (lo + hi) >> 1, j = k + 1 - i;
        if (i < a && j > 0 && dev_left(v, s, med, i) < dev_right(v, s, med, j - 1))
            lo = i + 1;
        else
            hi = i;
    }
    const int i = lo, j = k + 1 - lo;
    float x = -CUDART_INF_F;
    if (i > 0) x = dev_left(v, s, med, i - 1);
    if (j > 0) x = fmaxf(x, dev_right(v, s, med, j - 1));
    return x;
}

// One CTA per particle: the confidence of its n rescored hypotheses,
// (max - median) / (1.4826 (MAD + 1e-12)), MAD the median absolute
// deviation from the median.  nPow2 >= n is a power of two (shared floats).
// One sort: the deviations' median comes from the sorted values (dev_kth).
__global__ void __launch_bounds__(512)
k_peak_score(const float* __restrict__ dvp, int n, int nPow2, float* __restrict__ peak)
{
    extern __shared__ float v[];
    const float* d = dvp + (size_t)blockIdx.x * n;
    for (int i = threadIdx.x; i < nPow2; i += blockDim.x) v[i] = i < n ? d[i] : CUDART_INF_F;
    __syncthreads();
    bitonic_sort_asc(v, nPow2);
    if (threadIdx.x == 0) {
        const double med = sorted_median(v, n);
        const double mx = v[n - 1];
        float out = CUDART_NAN_F;
        if (!isnan(med) && !isnan(mx)) {
            // s: the first value not below the median
            int lo = 0, hi = n;
            while (lo < hi) {
                const int m = (lo + hi) >> 1;
                if ((double)v[m] < med) lo = m + 1;
                else hi = m;
            }
            const int s = lo;
            const double madv = (n & 1) ? (double)dev_kth(v, n, s, med, n / 2)
                                        : 0.5 * ((double)dev_kth(v, n, s, med, n / 2 - 1) +
                                                 (double)dev_kth(v, n, s, med, n / 2));
            out = (float)((mx - med) / (1.4826 * (madv + 1e-12)));
        }
        peak[blockIdx.x] = out;
    }
}

// First index of the largest of x[0 .. n) over a warp (lowest index on ties).
__device__ __forceinline__ int warp_argmax(const double* __restrict__ x, int n, int lane)
{
    double best = -CUDART_INF;
    int bi = 0x7fffffff;
    for (int j = lane; j < n; j += 32) {
        const double v = x[j];
        if (bi == 0x7fffffff || v > best) {
            best = v;
            bi = j;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    return bi;
}

// One warp per particle: the proposal's best rotation and translation
// (argmax of the marginals), its log-likelihood, and whether the particle
// falls back (confidence below peakMin, or not a number).
__global__ void k_best_proposal(const double* __restrict__ wR, const double* __restrict__ wT,
                                int nP, int nR, int nT, const double* __restrict__ quat,
                                const double* __restrict__ trans, const double* __restrict__ base,
                                const float* __restrict__ peak, float peakMin,
                                double* __restrict__ bestQuat, double* __restrict__ bestTrans,
                                double* __restrict__ bestBase, int* __restrict__ fellBack)
{
    const int l = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (l >= nP) return;
    const int r = warp_argmax(wR + (size_t)l * nR, nR, lane);
    const int t = warp_argmax(wT + (size_t)l * nT, nT, lane);
    if (lane < 4) bestQuat[4 * (size_t)l + lane] = quat[((size_t)l * nR + r) * 4 + lane];
    if (lane < 2) bestTrans[2 * (size_t)l + lane] = trans[((size_t)l * nT + t) * 2 + lane];
    if (lane == 0) {
        bestBase[l] = base[l];
        fellBack[l] = (peak[l] >= peakMin) ? 0 : 1;
    }
}

// Rows list[i] of src (w floats each) into row i of dst.
__global__ void k_gather_rows(const float* __restrict__ src, const int* __restrict__ list, int m,
                              int w, float* __restrict__ dst)
{
    const size_t n = (size_t)m * w;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t r = i / w, j = i - r * w;
        dst[i] = src[(size_t)list[r] * w + j];
    }
}

// One warp per fallback particle i: the global search's best rotation (a
// bank row) and translation, written to particle list[i]'s outputs.
__global__ void k_best_global(const double* __restrict__ gwR, const double* __restrict__ gwT,
                              const double* __restrict__ gbase, const int* __restrict__ list,
                              int m, int nB, int nTg, const double* __restrict__ bankQuat,
                              const double* __restrict__ gTrans, double* __restrict__ bestQuat,
                              double* __restrict__ bestTrans, double* __restrict__ bestBase)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= m) return;
    const int r = warp_argmax(gwR + (size_t)i * nB, nB, lane);
    const int t = warp_argmax(gwT + (size_t)i * nTg, nTg, lane);
    const int l = list[i];
    if (lane < 4) bestQuat[4 * (size_t)l + lane] = bankQuat[4 * (size_t)r + lane];
    if (lane < 2) bestTrans[2 * (size_t)l + lane] = gTrans[2 * (size_t)t + lane];
    if (lane == 0) bestBase[l] = gbase[i];
}

inline int grid_for(size_t n, int threads)
{
    return (int)std::min<size_t>((n + threads - 1) / threads, 152 * 32);
}

template <class T>
int copy_out(T* dst, const T* src, size_t n, cudaStream_t s)
{
    if (dst) TG3_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDeviceToDevice, s));
    return TG3_OK;
}

}  // namespace

}  // namespace tg3

using namespace tg3;

extern "C" int tg3_ctx_set_references(tg3_ctx* c, int cls, const float* emb, int n)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses) return fail(TG3_ERR_ARG, "class out of range");
    Bank& b = c->bank[cls];
    if (b.nB <= 0) return fail(TG3_ERR_STATE, "the class has no projection bank");
    if (!emb || n != b.nB)
        return fail(TG3_ERR_ARG, "references must match the bank's rotations one for one");
    if (!b.emb) TG3_CUDA(cudaMalloc(&b.emb, sizeof(float) * kEmbDim * (size_t)b.nB));
    TG3_CUDA(cudaMemcpyAsync(b.emb, emb, sizeof(float) * kEmbDim * (size_t)n,
                             cudaMemcpyDeviceToDevice, c->stream));
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    b.nEmb = n;
    return TG3_OK;
}

// The learned E-step; with dataReady, the compute stream waits for that
// event before the first kernel that reads dat, ctf or sigRcp (the
// host-buffer entry copies them on its copy stream meanwhile).
static int learned_expect(tg3_ctx* c, tg3_cnn* net, int nP, const float* images,
                          const float* dat, const float* ctf, const float* sigRcp,
                          const int* cls, int nRot, int nTrans, unsigned long long seed,
                          const double* gTrans, int nTg, float peakMin, int precision,
                          const tg3_learned_out* out, cudaEvent_t dataReady);

extern "C" int tg3_learned_expect_d(tg3_ctx* c, tg3_cnn* net, int nP, const float* images,
                                    const float* dat, const float* ctf, const float* sigRcp,
                                    const int* cls, int nRot, int nTrans,
                                    unsigned long long seed, const double* gTrans, int nTg,
                                    float peakMin, int precision, const tg3_learned_out* out)
{
    return learned_expect(c, net, nP, images, dat, ctf, sigRcp, cls, nRot, nTrans, seed, gTrans,
                          nTg, peakMin, precision, out, nullptr);
}

static int learned_expect(tg3_ctx* c, tg3_cnn* net, int nP, const float* images,
                          const float* dat, const float* ctf, const float* sigRcp,
                          const int* cls, int nRot, int nTrans, unsigned long long seed,
                          const double* gTrans, int nTg, float peakMin, int precision,
                          const tg3_learned_out* out, cudaEvent_t dataReady)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!net || !images || !dat || !ctf || !sigRcp || !cls || !gTrans || !out)
        return fail(TG3_ERR_ARG, "null argument");
    if (!out->bestQuat || !out->bestTrans || !out->baseL)
        return fail(TG3_ERR_ARG, "bestQuat, bestTrans and baseL are required outputs");
    if (nP <= 0 || nRot <= 0 || nTrans <= 0 || nTg <= 0 || nTrans > 256 || nTg > 256)
        return fail(TG3_ERR_ARG, "bad learned E-step shape (nTrans, nTg <= 256)");
    if ((long long)nRot * nTrans > kMaxPeakN)
        return fail(TG3_ERR_ARG, "nRot x nTrans must not exceed 16384");
    if (precision != TG3_SCORE_FP32 && precision != TG3_SCORE_BF16X3)
        return fail(TG3_ERR_ARG, "unknown precision");
    bool anyBank = false, anyRef = false;
    if ((st = upload_bank_views(c, &anyBank, &anyRef))) return st;
    if (!anyRef)
        return fail(TG3_ERR_STATE, "no class has references on the active pixel set "
                                   "(tg3_ctx_set_bank, then tg3_ctx_set_references)");
    int maxRef = 0, maxB = 0;
    for (int k = 0; k < kMaxClasses; k++) {
        const Bank& b = c->bank[k];
        if (b.nB > 0 && b.gen == c->px.gen && b.K == c->px.K) {
            maxB = std::max(maxB, b.nB);
            if (b.emb && b.nEmb == b.nB) maxRef = std::max(maxRef, b.nEmb);
        }
    }
    if (nRot > maxRef) return fail(TG3_ERR_ARG, "nRot exceeds the classes' reference counts");
    const int K = c->px.K;
    cudaStream_t s = c->stream;
    // ---- workspace
    Arena ar(c, WS_LEARN);
    const size_t oOut = ar.add(sizeof(float) * kNetOut * (size_t)nP),
                 oIdx = ar.add(sizeof(int) * (size_t)nP * nRot),
                 oQ = ar.add(sizeof(double) * 4 * (size_t)nP * nRot),
                 oT = ar.add(sizeof(double) * 2 * (size_t)nP * nTrans),
                 oPR = ar.add(sizeof(double) * (size_t)nP * nRot),
                 oPT = ar.add(sizeof(double) * (size_t)nP * nTrans),
                 oPC = ar.add(sizeof(double) * (size_t)nP),
                 oWC = ar.add(sizeof(double) * (size_t)nP),
                 oWR = ar.add(sizeof(double) * (size_t)nP * nRot),
                 oWT = ar.add(sizeof(double) * (size_t)nP * nTrans),
                 oB = ar.add(sizeof(double) * (size_t)nP),
                 oDvp = ar.add(sizeof(float) * (size_t)nP * nRot * nTrans),
                 oPk = ar.add(sizeof(float) * (size_t)nP),
                 oFb = ar.add(sizeof(int) * (size_t)nP),
                 oList = ar.add(sizeof(int) * (size_t)nP),
                 oGd = ar.add(sizeof(float) * 2 * (size_t)nP * K),
                 oGc = ar.add(sizeof(float) * (size_t)nP * K),
                 oGs = ar.add(sizeof(float) * (size_t)nP * K),
                 oGwC = ar.add(sizeof(double) * (size_t)nP),
                 oGwR = ar.add(sizeof(double) * (size_t)nP * std::max(maxB, 1)),
                 oGwT = ar.add(sizeof(double) * (size_t)nP * nTg),
                 oGb = ar.add(sizeof(double) * (size_t)nP),
                 oGpR = ar.add(sizeof(double) * (size_t)std::max(maxB, 1)),
                 oGpT = ar.add(sizeof(double) * (size_t)nTg);
    char* w = (char*)ws_get(c, WS_LEARN, ar.used, &st);
    if (!w) return st;
    float* net68 = (float*)(w + oOut);
    int* idx = (int*)(w + oIdx);
    double* quat = (double*)(w + oQ);
    double* trans = (double*)(w + oT);
    double* pwR = (double*)(w + oPR);
    double* pwT = (double*)(w + oPT);
    double* pwC = (double*)(w + oPC);
    double* wC = (double*)(w + oWC);
    double* wR = (double*)(w + oWR);
    double* wT = (double*)(w + oWT);
    double* base = (double*)(w + oB);
    float* dvp = (float*)(w + oDvp);
    float* peak = (float*)(w + oPk);
    int* fb = (int*)(w + oFb);
    int* list = (int*)(w + oList);
    float* gdat = (float*)(w + oGd);
    float* gctf = (float*)(w + oGc);
    float* gsig = (float*)(w + oGs);
    double* gwC = (double*)(w + oGwC);
    double* gwR = (double*)(w + oGwR);
    double* gwT = (double*)(w + oGwT);
    double* gbase = (double*)(w + oGb);
    double* gpR = (double*)(w + oGpR);
    double* gpT = (double*)(w + oGpT);
    // ---- 1-2: network and matching proposals
    {
        StageTimer tm(c, TG3_STAGE_NETWORK);
        // the network runs on its own stream: the inputs queued on ours first
        TG3_CUDA(cudaStreamSynchronize(s));
        if ((st = tg3_cnn_infer(net, images, nP, net68))) return st;
        TG3_CUDA(launch_match_propose_classes(net68, nP, c->d_refTable, cls, maxRef, nRot,
                                              nTrans, seed, quat, trans, idx, s));
    }
    k_fill_f64<<<grid_for((size_t)nP * nRot, 256), 256, 0, s>>>(pwR, (size_t)nP * nRot,
                                                                1.0 / nRot);
    k_fill_f64<<<grid_for((size_t)nP * nTrans, 256), 256, 0, s>>>(pwT, (size_t)nP * nTrans,
                                                                  1.0 / nTrans);
    k_fill_f64<<<grid_for(nP, 256), 256, 0, s>>>(pwC, nP, 1.0);
    TG3_LAUNCH_CHECK("uniform priors");
    if (dataReady) TG3_CUDA(cudaStreamWaitEvent(s, dataReady, 0));
    // ---- 3: exact rescoring from the banks
    if ((st = tg3_local_phase_bank_d(c, nP, nRot, nTrans, dat, ctf, sigRcp, idx, trans, pwR, pwT,
                                     pwC, cls, wC, wR, wT, base, dvp, precision)))
        return st;
    // ---- 4: confidence, the proposal's best pose, the fallback decision
    {
        StageTimer tm(c, TG3_STAGE_NETWORK);
        const int n = nRot * nTrans;
        int p2 = 1;
        while (p2 < n) p2 <<= 1;
        const size_t smem = sizeof(float) * p2;
        TG3_CUDA(cudaFuncSetAttribute(k_peak_score, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
        k_peak_score<<<nP, 512, smem, s>>>(dvp, n, p2, peak);
        TG3_LAUNCH_CHECK("proposal confidence");
        k_best_proposal<<<(nP + 7) / 8, 256, 0, s>>>(wR, wT, nP, nRot, nTrans, quat, trans, base,
                                                     peak, peakMin, out->bestQuat,
                                                     out->bestTrans, out->baseL, fb);
        TG3_LAUNCH_CHECK("proposal best pose");
    }
    // ---- 5: the fallback particles, class by class, against the global search
    std::vector<int> hFb(nP), hCls(nP);
    TG3_CUDA(cudaMemcpyAsync(hFb.data(), fb, sizeof(int) * nP, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(hCls.data(), cls, sizeof(int) * nP, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaStreamSynchronize(s));
    std::vector<int> hList;
    std::vector<std::pair<int, std::pair<int, int>>> groups;   // class, (start, count)
    for (int k = 0; k < kMaxClasses; k++) {
        const int start = (int)hList.size();
        for (int l = 0; l < nP; l++)
            if (hFb[l] && hCls[l] == k) hList.push_back(l);
        const int m = (int)hList.size() - start;
        if (m > 0) groups.push_back({k, {start, m}});
    }
    for (int l = 0; l < nP; l++)
        if (hFb[l] && (hCls[l] < 0 || hCls[l] >= kMaxClasses))
            return fail(TG3_ERR_ARG, "a particle's class is out of range");
    if (!hList.empty()) {
        StageTimer tm(c, TG3_STAGE_FALLBACK);
        c->fallbackScope = true;
        TG3_CUDA(cudaMemcpyAsync(list, hList.data(), sizeof(int) * hList.size(),
                                 cudaMemcpyHostToDevice, s));
        k_fill_f64<<<1, 256, 0, s>>>(gpT, nTg, 1.0 / nTg);
        for (const auto& g : groups) {
            const int k = g.first, start = g.second.first, m = g.second.second;
            const Bank& b = c->bank[k];
            if (b.nB <= 0 || b.gen != c->px.gen || b.K != K) {
                c->fallbackScope = false;
                return fail(TG3_ERR_STATE, "a fallback particle's class has no bank");
            }
            const int* li = list + start;
            k_gather_rows<<<grid_for((size_t)m * 2 * K, 256), 256, 0, s>>>(dat, li, m, 2 * K,
                                                                           gdat);
            k_gather_rows<<<grid_for((size_t)m * K, 256), 256, 0, s>>>(ctf, li, m, K, gctf);
            k_gather_rows<<<grid_for((size_t)m * K, 256), 256, 0, s>>>(sigRcp, li, m, K, gsig);
            k_fill_f64<<<grid_for(b.nB, 256), 256, 0, s>>>(gpR, b.nB, 1.0 / b.nB);
            TG3_LAUNCH_CHECK("fallback inputs");
            st = global_scan_bank(c, k, m, nTg, gdat, gctf, gsig, gTrans, gpR, gpT, gwC, gwR, gwT,
                                  gbase, nullptr, precision);
            if (st) {
                c->fallbackScope = false;
                return st;
            }
            k_best_global<<<(m + 7) / 8, 256, 0, s>>>(gwR, gwT, gbase, li, m, b.nB, nTg, b.quat,
                                                      gTrans, out->bestQuat, out->bestTrans,
                                                      out->baseL);
            TG3_LAUNCH_CHECK("fallback best pose");
        }
        c->fallbackScope = false;
    }
    // ---- optional outputs
    if ((st = copy_out(out->peak, peak, nP, s))) return st;
    if ((st = copy_out(out->fellBack, fb, nP, s))) return st;
    if ((st = copy_out(out->propIdx, idx, (size_t)nP * nRot, s))) return st;
    if ((st = copy_out(out->propQuat, quat, (size_t)nP * nRot * 4, s))) return st;
    if ((st = copy_out(out->propTrans, trans, (size_t)nP * nTrans * 2, s))) return st;
    if ((st = copy_out(out->propWR, wR, (size_t)nP * nRot, s))) return st;
    if ((st = copy_out(out->propWT, wT, (size_t)nP * nTrans, s))) return st;
    if ((st = copy_out(out->propBase, base, (size_t)nP, s))) return st;
    if ((st = copy_out(out->propDvp, dvp, (size_t)nP * nRot * nTrans, s))) return st;
    return tg3_ctx_sync(c);
}

extern "C" int tg3_ExpectLearned3D(tg3_ctx* c, tg3_cnn* net, int nP, const float* images,
                                   const float* dat, const float* ctf, const float* sigRcp,
                                   const int* cls, int nRot, int nTrans, unsigned long long seed,
                                   const double* gTrans, int nTg, float peakMin, int precision,
                                   double* bestQuat, double* bestTrans, double* baseL,
                                   float* peak, int* fellBack)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!images || !dat || !ctf || !sigRcp || !cls || !gTrans || !bestQuat || !bestTrans ||
        !baseL)
        return fail(TG3_ERR_ARG, "null host buffer");
    if (nP <= 0 || nTg <= 0) return fail(TG3_ERR_ARG, "bad batch shape");
    const int K = c->px.K;
    if (K <= 0) return fail(TG3_ERR_STATE, "pixel list not set");
    cudaStream_t s = c->stream;
    Arena ar(c, WS_LEARN_IO);
    const size_t oIm = ar.add(sizeof(float) * 64 * 64 * (size_t)nP),
                 oD = ar.add(sizeof(float) * 2 * (size_t)nP * K),
                 oC = ar.add(sizeof(float) * (size_t)nP * K),
                 oS = ar.add(sizeof(float) * (size_t)nP * K), oK = ar.add(sizeof(int) * nP),
                 oG = ar.add(sizeof(double) * 2 * (size_t)nTg),
                 oQ = ar.add(sizeof(double) * 4 * (size_t)nP),
                 oT = ar.add(sizeof(double) * 2 * (size_t)nP),
                 oB = ar.add(sizeof(double) * (size_t)nP), oP = ar.add(sizeof(float) * nP),
                 oF = ar.add(sizeof(int) * nP);
    char* w = (char*)ws_get(c, WS_LEARN_IO, ar.used, &st);
    if (!w) return st;
    const auto h2d = [&](size_t off, const void* src, size_t bytes, cudaStream_t on) {
        return cudaMemcpyAsync(w + off, src, bytes, cudaMemcpyHostToDevice, on);
    };
    // the images, classes and translations on the compute stream (the
    // network needs them first); the data, CTFs and weights, nine tenths of
    // the bytes, on the copy stream while the network and the matching run
    if (!c->copyStream) TG3_CUDA(cudaStreamCreateWithFlags(&c->copyStream, cudaStreamNonBlocking));
    if (!c->copyDone) TG3_CUDA(cudaEventCreateWithFlags(&c->copyDone, cudaEventDisableTiming));
    TG3_CUDA(h2d(oIm, images, sizeof(float) * 64 * 64 * (size_t)nP, s));
    TG3_CUDA(h2d(oK, cls, sizeof(int) * nP, s));
    TG3_CUDA(h2d(oG, gTrans, sizeof(double) * 2 * (size_t)nTg, s));
    // the copy stream does not overwrite the arena before the compute
    // stream's earlier work on it is done
    TG3_CUDA(cudaEventRecord(c->copyDone, s));
    {
        // a failure part-way leaves no copy still landing in the arena
        cudaError_t e = cudaStreamWaitEvent(c->copyStream, c->copyDone, 0);
        if (e == cudaSuccess) e = h2d(oD, dat, sizeof(float) * 2 * (size_t)nP * K, c->copyStream);
        if (e == cudaSuccess) e = h2d(oC, ctf, sizeof(float) * (size_t)nP * K, c->copyStream);
        if (e == cudaSuccess) e = h2d(oS, sigRcp, sizeof(float) * (size_t)nP * K, c->copyStream);
        if (e == cudaSuccess) e = cudaEventRecord(c->copyDone, c->copyStream);
        if (e != cudaSuccess) {
            cudaStreamSynchronize(c->copyStream);
            return cuda_fail(e, "learned E-step input copies");
        }
    }
    tg3_learned_out o = {};
    o.bestQuat = (double*)(w + oQ);
    o.bestTrans = (double*)(w + oT);
    o.baseL = (double*)(w + oB);
    o.peak = (float*)(w + oP);
    o.fellBack = (int*)(w + oF);
    st = learned_expect(c, net, nP, (const float*)(w + oIm), (const float*)(w + oD),
                        (const float*)(w + oC), (const float*)(w + oS), (const int*)(w + oK), nRot,
                        nTrans, seed, (const double*)(w + oG), nTg, peakMin, precision, &o,
                        c->copyDone);
    if (st) {
        // the copies may still be landing in the arena: let them finish
        cudaStreamSynchronize(c->copyStream);
        return st;
    }
    TG3_CUDA(cudaMemcpyAsync(bestQuat, o.bestQuat, sizeof(double) * 4 * nP,
                             cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(bestTrans, o.bestTrans, sizeof(double) * 2 * nP,
                             cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(baseL, o.baseL, sizeof(double) * nP, cudaMemcpyDeviceToHost, s));
    if (peak) TG3_CUDA(cudaMemcpyAsync(peak, o.peak, sizeof(float) * nP, cudaMemcpyDeviceToHost, s));
    if (fellBack)
        TG3_CUDA(cudaMemcpyAsync(fellBack, o.fellBack, sizeof(int) * nP, cudaMemcpyDeviceToHost,
                                 s));
    TG3_CUDA(cudaStreamSynchronize(s));
    return TG3_OK;
}
