// tg3_ragged.cu -- a batch of particles with uneven hypothesis sets as one
// replayable plan.
//
// After the filter's narrowing and resampling rounds every particle keeps its
// own number of rotations and translations (Particle::resample draws a count
// per particle, src/Particle.cpp:1275-1463) and belongs to one class, every
// class with its own pixel cutoff.  A plan covers one batch of such particles:
//   - particles are ordered by (class, rotations descending) and cut into
//     waves whose projection bank fits a byte budget;
//   - within a wave every particle is padded to the wave's largest rotation
//     and translation counts with copies of its own first rotation /
//     translation carrying zero prior weight.  A copy cannot raise the
//     maximum log-likelihood and adds +0 to every marginal sum, and the
//     resampler draws from the particle's own n entries only, so every
//     output equals that of the particle scored alone;
//   - per wave: k_ragged_gather builds the padded inputs, the batched local
//     phase scores them (tg3_local_phase_d), the resampler draws per-particle
//     counts, k_ragged_scatter writes the particles' own entries back;
//   - the whole sequence is captured once in a CUDA graph and replayed.
// The wave budget, the split cross term's K block and the projection's
// rotations per CTA are chosen per plan by an autotuner that times the
// candidates on the plan's own batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {

namespace {

struct RaggedIn {
    // packed per particle: pixel values at pixOff[l] (K of its class),
    // rotations at rOff[l], translations at tOff[l]
    const float2* dat;
    const float* ctf;
    const float* sig;
    const double* quat;
    const double* trans;
    const double* pwR;
    const double* pwT;
    const double* pwC;
    const int* permR;
    const double* u0R;
    const double* peakR;
    const int* permT;
    const double* u0T;
    const double* peakT;
};

struct RaggedOut {
    double* wC;
    double* base;
    double* wR;
    double* wT;
    int* srcR;
    double* wOutR;
    int* srcT;
    double* wOutT;
    int* topR;
    int* topT;
};

struct WaveBuf {
    float2* dat;
    float* ctf;
    float* sig;
    double* quat;
    double* trans;
    double* pwR;
    double* pwT;
    double* pwC;
    int* cls;
    int* permR;
    double* u0R;
    double* peakR;
    int* permT;
    double* u0T;
    double* peakT;
    int* nPerR;
    int* nPerT;
    double* wC;
    double* base;
    double* wR;
    double* wT;
    int* srcR;
    double* wOutR;
    int* srcT;
    double* wOutT;
    int* topR;
    int* topT;
};

// One CTA per wave slot i: particle l = idx[i] padded to nRw rotations and
// nTw translations.
__global__ void k_ragged_gather(const int* __restrict__ idx, int K, int nRw, int nTw,
                                const long long* __restrict__ pixOff,
                                const long long* __restrict__ rOff,
                                const long long* __restrict__ tOff, const int* __restrict__ cls,
                                const int* __restrict__ nR, const int* __restrict__ nT,
                                RaggedIn in, WaveBuf wb)
{
    const int i = blockIdx.x;
    const int l = idx[i];
    const long long po = pixOff[l], ro = rOff[l], to = tOff[l];
    const int nr = nR[l], nt = nT[l];
    for (int p = threadIdx.x; p < K; p += blockDim.x) {
        wb.dat[(size_t)i * K + p] = in.dat[po + p];
        wb.ctf[(size_t)i * K + p] = in.ctf[po + p];
        wb.sig[(size_t)i * K + p] = in.sig[po + p];
    }
    for (int r = threadIdx.x; r < nRw; r += blockDim.x) {
        const bool v = r < nr;
        const long long s = ro + (v ? r : 0);
        for (int k = 0; k < 4; k++) wb.quat[((size_t)i * nRw + r) * 4 + k] = in.quat[s * 4 + k];
        wb.pwR[(size_t)i * nRw + r] = v ? in.pwR[s] : 0.0;
        wb.permR[(size_t)i * nRw + r] = v ? in.permR[s] : r;
    }
    for (int t = threadIdx.x; t < nTw; t += blockDim.x) {
        const bool v = t < nt;
        const long long s = to + (v ? t : 0);
        for (int k = 0; k < 2; k++) wb.trans[((size_t)i * nTw + t) * 2 + k] = in.trans[s * 2 + k];
        wb.pwT[(size_t)i * nTw + t] = v ? in.pwT[s] : 0.0;
        wb.permT[(size_t)i * nTw + t] = v ? in.permT[s] : t;
    }
    if (threadIdx.x == 0) {
        wb.pwC[i] = in.pwC[l];
        wb.cls[i] = cls[l];
        wb.u0R[i] = in.u0R[l];
        wb.peakR[i] = in.peakR[l];
        wb.u0T[i] = in.u0T[l];
        wb.peakT[i] = in.peakT[l];
        wb.nPerR[i] = nr;
        wb.nPerT[i] = nt;
    }
}

// The particles' own entries of a wave back into the packed outputs.
__global__ void k_ragged_scatter(const int* __restrict__ idx, int nRw, int nTw,
                                 const long long* __restrict__ rOff,
                                 const long long* __restrict__ tOff, const int* __restrict__ nR,
                                 const int* __restrict__ nT, WaveBuf wb, RaggedOut out)
{
    const int i = blockIdx.x;
    const int l = idx[i];
    const long long ro = rOff[l], to = tOff[l];
    const int nr = nR[l], nt = nT[l];
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        out.wR[ro + r] = wb.wR[(size_t)i * nRw + r];
        out.srcR[ro + r] = wb.srcR[(size_t)i * nRw + r];
        out.wOutR[ro + r] = wb.wOutR[(size_t)i * nRw + r];
    }
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        out.wT[to + t] = wb.wT[(size_t)i * nTw + t];
        out.srcT[to + t] = wb.srcT[(size_t)i * nTw + t];
        out.wOutT[to + t] = wb.wOutT[(size_t)i * nTw + t];
    }
    if (threadIdx.x == 0) {
        out.wC[l] = wb.wC[i];
        out.base[l] = wb.base[i];
        out.topR[l] = wb.topR[i];
        out.topT[l] = wb.topT[i];
    }
}

struct Wave {
    int cls, first, w, nR, nT;
};

}  // namespace
}  // namespace tg3

using namespace tg3;

struct tg3_plan {
    tg3_ctx* c = nullptr;
    int nP = 0, precision = 0;
    size_t budget = 0;
    int bk = 64;                 // the local phase's K block (TG3_OPT_LOCAL_BK) for this plan
    int pg = 8;                  // the projection's rotations per CTA (TG3_OPT_PROJECT_GROUP)
    RaggedIn in;
    RaggedOut out;
    std::vector<int> clsH, nRH, nTH;
    std::vector<Wave> waves;
    // device: per-particle shapes and offsets, the waves' particle lists
    int* dCls = nullptr;
    int* dNR = nullptr;
    int* dNT = nullptr;
    long long* dPixOff = nullptr;
    long long* dROff = nullptr;
    long long* dTOff = nullptr;
    int* dIdx = nullptr;
    void* waveMem = nullptr;
    WaveBuf wb;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

void plan_free_waves(tg3_plan* p)
{
    cudaFree(p->dIdx);
    cudaFree(p->waveMem);
    p->dIdx = nullptr;
    p->waveMem = nullptr;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
}

// Cut the batch into waves for a projection-bank budget and size the wave
// buffers for the largest of them.
int plan_waves(tg3_plan* p, size_t budget)
{
    tg3_ctx* c = p->c;
    plan_free_waves(p);
    p->budget = budget;
    std::vector<int> order(p->nP);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (p->clsH[a] != p->clsH[b]) return p->clsH[a] < p->clsH[b];
        return p->nRH[a] > p->nRH[b];
    });
    p->waves.clear();
    size_t maxK = 0, maxRows = 0, maxTr = 0, maxW = 0;
    for (int i = 0; i < p->nP;) {
        const int cl = p->clsH[order[i]];
        const size_t Kp = (size_t)c->pxSlot[cl].Kp;
        Wave w{cl, i, 0, p->nRH[order[i]], 0};
        while (i < p->nP && p->clsH[order[i]] == cl) {
            const size_t rows = (size_t)(w.w + 1) * w.nR;
            if (w.w > 0 && (rows * Kp * sizeof(float) > budget || w.w >= 65535)) break;
            w.nT = std::max(w.nT, p->nTH[order[i]]);
            w.w++;
            i++;
        }
        p->waves.push_back(w);
        maxK = std::max(maxK, (size_t)c->pxSlot[cl].K);
        maxRows = std::max(maxRows, (size_t)w.w * w.nR);
        maxTr = std::max(maxTr, (size_t)w.w * w.nT);
        maxW = std::max(maxW, (size_t)w.w);
    }
    TG3_CUDA(cudaMalloc(&p->dIdx, sizeof(int) * p->nP));
    TG3_CUDA(cudaMemcpy(p->dIdx, order.data(), sizeof(int) * p->nP, cudaMemcpyHostToDevice));
    // wave buffers, one allocation
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += round_up(bytes, 256);
        return o;
    };
    const size_t oDat = take(sizeof(float2) * maxW * maxK), oCtf = take(sizeof(float) * maxW * maxK),
                 oSig = take(sizeof(float) * maxW * maxK), oQuat = take(sizeof(double) * 4 * maxRows),
                 oTrans = take(sizeof(double) * 2 * maxTr), oPwR = take(sizeof(double) * maxRows),
                 oPwT = take(sizeof(double) * maxTr), oPwC = take(sizeof(double) * maxW),
                 oCls = take(sizeof(int) * maxW), oPermR = take(sizeof(int) * maxRows),
                 oU0R = take(sizeof(double) * maxW), oPeakR = take(sizeof(double) * maxW),
                 oPermT = take(sizeof(int) * maxTr), oU0T = take(sizeof(double) * maxW),
                 oPeakT = take(sizeof(double) * maxW), oNR = take(sizeof(int) * maxW),
                 oNT = take(sizeof(int) * maxW), oWC = take(sizeof(double) * maxW),
                 oBase = take(sizeof(double) * maxW), oWR = take(sizeof(double) * maxRows),
                 oWT = take(sizeof(double) * maxTr), oSrcR = take(sizeof(int) * maxRows),
                 oWOutR = take(sizeof(double) * maxRows), oSrcT = take(sizeof(int) * maxTr),
                 oWOutT = take(sizeof(double) * maxTr), oTopR = take(sizeof(int) * maxW),
                 oTopT = take(sizeof(int) * maxW);
    TG3_CUDA(cudaMalloc(&p->waveMem, off));
    char* m = static_cast<char*>(p->waveMem);
    WaveBuf& b = p->wb;
    b.dat = (float2*)(m + oDat);
    b.ctf = (float*)(m + oCtf);
    b.sig = (float*)(m + oSig);
    b.quat = (double*)(m + oQuat);
    b.trans = (double*)(m + oTrans);
    b.pwR = (double*)(m + oPwR);
    b.pwT = (double*)(m + oPwT);
    b.pwC = (double*)(m + oPwC);
    b.cls = (int*)(m + oCls);
    b.permR = (int*)(m + oPermR);
    b.u0R = (double*)(m + oU0R);
    b.peakR = (double*)(m + oPeakR);
    b.permT = (int*)(m + oPermT);
    b.u0T = (double*)(m + oU0T);
    b.peakT = (double*)(m + oPeakT);
    b.nPerR = (int*)(m + oNR);
    b.nPerT = (int*)(m + oNT);
    b.wC = (double*)(m + oWC);
    b.base = (double*)(m + oBase);
    b.wR = (double*)(m + oWR);
    b.wT = (double*)(m + oWT);
    b.srcR = (int*)(m + oSrcR);
    b.wOutR = (double*)(m + oWOutR);
    b.srcT = (int*)(m + oSrcT);
    b.wOutT = (double*)(m + oWOutT);
    b.topR = (int*)(m + oTopR);
    b.topT = (int*)(m + oTopT);
    return TG3_OK;
}

// The launches of every wave, in order, on the context stream.
int plan_issue_waves(tg3_plan* p);

// The plan's waves with its K block and projection group set on the context
// for their duration.
int plan_issue(tg3_plan* p)
{
    const int saved = p->c->localBK, savedG = p->c->projGroup;
    p->c->localBK = p->bk;
    p->c->projGroup = p->pg;
    const int st = plan_issue_waves(p);
    p->c->localBK = saved;
    p->c->projGroup = savedG;
    return st;
}

int plan_issue_waves(tg3_plan* p)
{
    tg3_ctx* c = p->c;
    cudaStream_t s = c->stream;
    int st;
    for (const Wave& w : p->waves) {
        if ((st = tg3_ctx_use_pixels(c, w.cls))) return st;
        const int K = c->px.K;
        k_ragged_gather<<<w.w, 256, 0, s>>>(p->dIdx + w.first, K, w.nR, w.nT, p->dPixOff, p->dROff,
                                             p->dTOff, p->dCls, p->dNR, p->dNT, p->in, p->wb);
        TG3_LAUNCH_CHECK("ragged gather");
        if ((st = tg3_local_phase_d(c, w.w, w.nR, w.nT, reinterpret_cast<const float*>(p->wb.dat),
                                    p->wb.ctf, p->wb.sig, p->wb.quat, p->wb.trans, p->wb.pwR,
                                    p->wb.pwT, p->wb.pwC, p->wb.cls, p->wb.wC, p->wb.wR, p->wb.wT,
                                    p->wb.base, nullptr, p->precision)))
            return st;
        TG3_CUDA(launch_resample(w.w, w.nR, p->wb.wR, p->wb.pwR, p->wb.permR, p->wb.u0R,
                                 p->wb.peakR, w.nR, p->wb.srcR, p->wb.wOutR, p->wb.topR, c->d_flag,
                                 s, p->wb.nPerR));
        TG3_CUDA(launch_resample(w.w, w.nT, p->wb.wT, p->wb.pwT, p->wb.permT, p->wb.u0T,
                                 p->wb.peakT, w.nT, p->wb.srcT, p->wb.wOutT, p->wb.topT, c->d_flag,
                                 s, p->wb.nPerT));
        k_ragged_scatter<<<w.w, 256, 0, s>>>(p->dIdx + w.first, w.nR, w.nT, p->dROff, p->dTOff,
                                              p->dNR, p->dNT, p->wb, p->out);
        TG3_LAUNCH_CHECK("ragged scatter");
    }
    // leave the context's own pixel set active again
    if (c->pxMain.iCol) c->px = c->pxMain;
    return TG3_OK;
}

// Eager run, synchronised; milliseconds of the launches.
int plan_time(tg3_plan* p, float* ms)
{
    tg3_ctx* c = p->c;
    cudaEvent_t e0, e1;
    TG3_CUDA(cudaEventCreate(&e0));
    TG3_CUDA(cudaEventCreate(&e1));
    TG3_CUDA(cudaEventRecord(e0, c->stream));
    int st = plan_issue(p);
    TG3_CUDA(cudaEventRecord(e1, c->stream));
    TG3_CUDA(cudaEventSynchronize(e1));
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    return tg3_ctx_sync(c);
}

}  // namespace

extern "C" int tg3_ragged_plan_create(
    tg3_ctx* c, int nP, const int* cls, const int* nR, const int* nT, const float* dat,
    const float* ctf, const float* sigRcp, const double* quat, const double* trans,
    const double* pwR, const double* pwT, const double* pwC, const int* permR, const double* u0R,
    const double* peakR, const int* permT, const double* u0T, const double* peakT, double* wC,
    double* baseL, double* wR, double* wT, int* srcR, double* wOutR, int* srcT, double* wOutT,
    int* topR, int* topT, int precision, size_t budget, int use_graph, tg3_plan** out)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!out || nP <= 0 || !cls || !nR || !nT) return fail(TG3_ERR_ARG, "bad plan arguments");
    if (!dat || !ctf || !sigRcp || !quat || !trans || !pwR || !pwT || !pwC || !permR || !u0R ||
        !peakR || !permT || !u0T || !peakT || !wC || !baseL || !wR || !wT || !srcR || !wOutR ||
        !srcT || !wOutT || !topR || !topT)
        return fail(TG3_ERR_ARG, "null device pointer");
    std::vector<long long> pixOff(nP), rOff(nP), tOff(nP);
    long long pk = 0, rk = 0, tk = 0;
    for (int l = 0; l < nP; l++) {
        if (cls[l] < 0 || cls[l] >= kMaxClasses || !c->pxSlot[cls[l]].iCol)
            return fail(TG3_ERR_STATE, "no pixel slot for a particle's class");
        if (!c->vol[cls[l]].blocks) return fail(TG3_ERR_STATE, "no volume for a particle's class");
        if (nR[l] <= 0 || nT[l] <= 0) return fail(TG3_ERR_ARG, "empty hypothesis set");
        pixOff[l] = pk;
        rOff[l] = rk;
        tOff[l] = tk;
        pk += c->pxSlot[cls[l]].K;
        rk += nR[l];
        tk += nT[l];
    }
    tg3_plan* p = new tg3_plan();
    p->c = c;
    p->nP = nP;
    p->precision = precision;
    p->clsH.assign(cls, cls + nP);
    p->nRH.assign(nR, nR + nP);
    p->nTH.assign(nT, nT + nP);
    p->in = RaggedIn{reinterpret_cast<const float2*>(dat), ctf, sigRcp, quat, trans, pwR, pwT,
                     pwC, permR, u0R, peakR, permT, u0T, peakT};
    p->out = RaggedOut{wC, baseL, wR, wT, srcR, wOutR, srcT, wOutT, topR, topT};
    auto fail_free = [&](int code) {
        tg3_ragged_plan_destroy(p);
        return code;
    };
    if (cudaMalloc(&p->dCls, sizeof(int) * nP) != cudaSuccess ||
        cudaMalloc(&p->dNR, sizeof(int) * nP) != cudaSuccess ||
        cudaMalloc(&p->dNT, sizeof(int) * nP) != cudaSuccess ||
        cudaMalloc(&p->dPixOff, sizeof(long long) * nP) != cudaSuccess ||
        cudaMalloc(&p->dROff, sizeof(long long) * nP) != cudaSuccess ||
        cudaMalloc(&p->dTOff, sizeof(long long) * nP) != cudaSuccess)
        return fail_free(fail(TG3_ERR_ALLOC, "plan allocation"));
    cudaMemcpy(p->dCls, cls, sizeof(int) * nP, cudaMemcpyHostToDevice);
    cudaMemcpy(p->dNR, nR, sizeof(int) * nP, cudaMemcpyHostToDevice);
    cudaMemcpy(p->dNT, nT, sizeof(int) * nP, cudaMemcpyHostToDevice);
    cudaMemcpy(p->dPixOff, pixOff.data(), sizeof(long long) * nP, cudaMemcpyHostToDevice);
    cudaMemcpy(p->dROff, rOff.data(), sizeof(long long) * nP, cudaMemcpyHostToDevice);
    if (cudaMemcpy(p->dTOff, tOff.data(), sizeof(long long) * nP, cudaMemcpyHostToDevice) !=
        cudaSuccess)
        return fail_free(fail(TG3_ERR_CUDA, "plan upload"));
    const bool timing = c->timing;
    c->timing = false;
    p->bk = c->localBK;
    p->pg = c->projGroup;
    if (budget == 0) {
        // autotune: time every candidate (wave budget, and for the split
        // precision the cross term's K block: 128-byte stages of 64 bf16 or
        // 64-byte stages of 32) on this batch -- the first run of a candidate
        // also sizes the workspaces -- and keep the fastest
        const size_t cand[3] = {(size_t)2 << 30, (size_t)6 << 30, (size_t)16 << 30};
        const int bks[2] = {64, 32};
        const int nbk = precision == TG3_SCORE_BF16X3 ? 2 : 1;
        float best = 1e30f;
        size_t bestB = cand[0];
        int bestK = 64;
        for (size_t b : cand)
            for (int ik = 0; ik < nbk; ik++) {
                float ms = 0;
                p->bk = bks[ik];
                if ((st = plan_waves(p, b)) || (st = plan_time(p, &ms)) ||
                    (st = plan_time(p, &ms))) {
                    c->timing = timing;
                    return fail_free(st);
                }
                if (ms < best) {
                    best = ms;
                    bestB = b;
                    bestK = bks[ik];
                }
            }
        budget = bestB;
        p->bk = bestK;
        // then the projection's tile: rotations per CTA for each pixel chunk
        // (the other two of 4, 8, 16), at the chosen budget and K block
        if ((st = plan_waves(p, budget))) {
            c->timing = timing;
            return fail_free(st);
        }
        const int pg0 = p->pg;
        int bestG = pg0;
        for (int g : {4, 8, 16}) {
            if (g == pg0) continue;
            float ms = 0;
            p->pg = g;
            if ((st = plan_time(p, &ms)) || (st = plan_time(p, &ms))) {
                c->timing = timing;
                return fail_free(st);
            }
            if (ms < best) {
                best = ms;
                bestG = g;
            }
        }
        p->pg = bestG;
    }
    float warmMs = 0;
    if ((st = plan_waves(p, budget)) || (st = plan_time(p, &warmMs))) {
        c->timing = timing;
        return fail_free(st);
    }
    if (use_graph) {
        cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
            st = plan_issue(p);
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
            if (st || e2 != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                c->timing = timing;
                return fail_free(st ? st : cuda_fail(e2, "graph capture"));
            }
            p->graph = g;
            e = cudaGraphInstantiate(&p->exec, g, 0);
        }
        if (e != cudaSuccess) {
            c->timing = timing;
            return fail_free(cuda_fail(e, "graph instantiation"));
        }
    }
    c->timing = timing;
    *out = p;
    return TG3_OK;
}

extern "C" int tg3_ragged_plan_run(tg3_plan* p)
{
    if (!p) return fail(TG3_ERR_ARG, "null plan");
    if (p->exec) {
        TG3_CUDA(cudaGraphLaunch(p->exec, p->c->stream));
        return TG3_OK;
    }
    const bool timing = p->c->timing;
    p->c->timing = false;
    const int st = plan_issue(p);
    p->c->timing = timing;
    return st;
}

extern "C" int tg3_ragged_plan_info(const tg3_plan* p, int* waves, size_t* budget)
{
    if (!p) return fail(TG3_ERR_ARG, "null plan");
    if (waves) *waves = (int)p->waves.size();
    if (budget) *budget = p->budget;
    return TG3_OK;
}

extern "C" int tg3_ragged_plan_project_group(const tg3_plan* p, int* group)
{
    if (!p || !group) return fail(TG3_ERR_ARG, "null plan or output");
    *group = p->pg;
    return TG3_OK;
}

extern "C" int tg3_ragged_plan_kblock(const tg3_plan* p, int* bk)
{
    if (!p || !bk) return fail(TG3_ERR_ARG, "null plan or output");
    *bk = p->bk;
    return TG3_OK;
}

extern "C" int tg3_ragged_plan_destroy(tg3_plan* p)
{
    if (!p) return TG3_OK;
    if (p->c) cudaStreamSynchronize(p->c->stream);
    plan_free_waves(p);
    cudaFree(p->dCls);
    cudaFree(p->dNR);
    cudaFree(p->dNT);
    cudaFree(p->dPixOff);
    cudaFree(p->dROff);
    cudaFree(p->dTOff);
    delete p;
    return TG3_OK;
}
