// tg3_api.cu -- the extern "C" boundary of libtg3.so (include/thunder_gb300.h).
//
// Host orchestration only: argument checks, workspace management, staging of
// host buffers, and the kernel sequences of the E-step and the insertion.
// Every failure returns a status and records a message; nothing falls back to
// host computation.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tg3_internal.cuh"

namespace tg3 {

static thread_local std::string g_err;

void set_error(const std::string& msg) { g_err = msg; }

int fail(int status, const std::string& msg)
{
    g_err = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* what)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? TG3_ERR_ALLOC : TG3_ERR_CUDA;
}

void* ws_get(tg3_ctx* c, WsSlot s, size_t bytes, int* status)
{
    Buffer& b = c->ws[s];
    if (bytes == 0) bytes = 256;
    if (b.bytes < bytes) {
        if (b.ptr) {
            cudaStreamSynchronize(c->stream);
            cudaFree(b.ptr);
            b.ptr = nullptr;
            b.bytes = 0;
        }
        size_t want = round_up(bytes + bytes / 8, (size_t)2 << 20);
        cudaError_t e = cudaMalloc(&b.ptr, want);
        if (e != cudaSuccess) {
            b.ptr = nullptr;
            *status = cuda_fail(e, "workspace allocation");
            return nullptr;
        }
        b.bytes = want;
    }
    *status = TG3_OK;
    return b.ptr;
}

// ---------------------------------------------------------- stage timing --
static cudaEvent_t take_event(tg3_ctx* c)
{
    if (!c->eventPool.empty()) {
        cudaEvent_t e = c->eventPool.back();
        c->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

StageTimer::StageTimer(tg3_ctx* c_, int s) : c(c_), stage(s)
{
    if (!c->timing) return;
    if (c->fallbackScope) {
        if (s != TG3_STAGE_CROSS && s != TG3_STAGE_NORM) return;
        if (s == TG3_STAGE_CROSS) stage = TG3_STAGE_FALLBACK_CROSS;
    }
    a = take_event(c);
    b = take_event(c);
    if (a) cudaEventRecord(a, c->stream);
}

StageTimer::~StageTimer()
{
    if (!c->timing || !a || !b) return;
    cudaEventRecord(b, c->stream);
    c->pending[stage].emplace_back(a, b);
}

static void collect_times(tg3_ctx* c)
{
    for (int s = 0; s < TG3_STAGE_COUNT; s++) {
        for (auto& pr : c->pending[s]) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) {
                c->stageMs[s] += ms;
                c->stageLaunches[s] += 1;
            }
            c->eventPool.push_back(pr.first);
            c->eventPool.push_back(pr.second);
        }
        c->pending[s].clear();
    }
}

// ------------------------------------------------------------- MKB table --
// I0 from its power series sum_k ((x/2)^k / k!)^2 (Abramowitz & Stegun
// 9.6.10); MKB_FT_R2 order 0 (src/Functions/Functions.cpp:108-126) tabulated
// on n + 1 uniform r^2 points over [0, b] (TabFunction::init,
// src/TabFunction.cpp:25-39).
static double bessel_i0(double x)
{
    double q = 0.25 * x * x, term = 1, sum = 1;
    for (int k = 1; k < 200; k++) {
        term *= q / ((double)k * k);
        sum += term;
        if (term < sum * 1e-17) break;
    }
    return sum;
}

static void mkb_table(double a, double alpha, double b, int n, std::vector<float>& tab,
                      int& nz)
{
    const double s = b / n, i0a = bessel_i0(alpha);
    tab.assign(n + 1, 0.f);
    nz = 0;
    for (int i = 0; i <= n; i++) {
        const double u2 = (i * s) / (a * a);
        double v = u2 > 1 ? 0.0 : bessel_i0(alpha * std::sqrt(1 - u2)) / i0a;
        tab[i] = (float)v;
        if (v != 0.0) nz = i;
    }
}

constexpr double kMkbA = 1.9, kMkbAlpha = 15.0;
constexpr int kMkbN = 100000;

int check_ctx(tg3_ctx* c)
{
    if (!c) return fail(TG3_ERR_ARG, "null context");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return TG3_OK;
}

// Every rotated pixel must stay inside the stored half volume, |R v| = |v|:
// margin 1 keeps a trilinear sample's corner block (its x0 + 1 <= vdim / 2
// is stored; its y0, z0 stay in [-vdim / 2, vdim / 2)), margin 2 also the
// MKB insertion support.
int check_geometry(tg3_ctx* c, int vdim, int pf, double margin)
{
    if (c->px.K <= 0) return fail(TG3_ERR_STATE, "pixel list not set");
    if (c->px.maxRadius * pf + margin > vdim / 2)
        return fail(TG3_ERR_ARG, "pixel radius " + std::to_string(c->px.maxRadius) +
                                     " x pf does not fit the volume edge " + std::to_string(vdim));
    return TG3_OK;
}

// The weights kernel keeps 2 nT floats in shared memory.
static int check_weights_shape(int nR, int nT)
{
    if (nR <= 0 || (size_t)2 * nT * sizeof(float) > 48 * 1024)
        return fail(TG3_ERR_UNSUPPORTED, "nT must not exceed 6144");
    return TG3_OK;
}

static int sync_and_check(tg3_ctx* c)
{
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    int flag = 0;
    TG3_CUDA(cudaMemcpy(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        TG3_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
        if (flag & 1) return fail(TG3_ERR_ARG, "resampling permutation out of range");
        if (flag & 2) return fail(TG3_ERR_NUMERIC, "resampling weights sum to zero");
        if (flag & 4) return fail(TG3_ERR_TIMEOUT, "device wait expired");
        if (flag & 8) return fail(TG3_ERR_STATE, "a particle's class has no volume set");
        if (flag & (1 << 16))
            return fail(TG3_ERR_ARG, "bank index out of range (or its class has no bank on the "
                                     "active pixel set)");
        return fail(TG3_ERR_CUDA, "device error flag " + std::to_string(flag));
    }
    return TG3_OK;
}

// Per-device default context used by the reference-shaped entry points.
static tg3_ctx* default_ctx(int* status)
{
    static std::mutex mu;
    static tg3_ctx* ctxs[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *status = cuda_fail(e, "cudaGetDevice");
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 0 || dev >= 64) {
        *status = fail(TG3_ERR_ARG, "device ordinal out of range");
        return nullptr;
    }
    if (!ctxs[dev]) {
        tg3_ctx* c = nullptr;
        *status = tg3_ctx_create(&c, dev);
        if (*status != TG3_OK) return nullptr;
        ctxs[dev] = c;
    }
    *status = TG3_OK;
    return ctxs[dev];
}

template <class T>
static int upload(tg3_ctx* c, WsSlot slot, size_t offset_bytes, const T* host, size_t n,
                  T** dev)
{
    int st = TG3_OK;
    char* base = (char*)ws_get(c, slot, offset_bytes + n * sizeof(T), &st);
    if (!base) return st;
    *dev = reinterpret_cast<T*>(base + offset_bytes);
    if (n) TG3_CUDA(cudaMemcpyAsync(*dev, host, n * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return TG3_OK;
}


}  // namespace tg3

using namespace tg3;

// ===================================================================== misc
extern "C" const char* tg3_status_string(int s)
{
    switch (s) {
    case TG3_OK: return "ok";
    case TG3_ERR_ARG: return "invalid argument";
    case TG3_ERR_CUDA: return "CUDA error";
    case TG3_ERR_ALLOC: return "allocation failed";
    case TG3_ERR_STATE: return "call out of order";
    case TG3_ERR_TIMEOUT: return "device wait expired";
    case TG3_ERR_NUMERIC: return "numeric failure";
    case TG3_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

extern "C" const char* tg3_last_error(void) { return g_err.c_str(); }

extern "C" const char* tg3_version(void) { return "tg3 1.0 sm_103a"; }

extern "C" int tg3_getAviDevice(int* gpus, int cap, int* n)
{
    if (!n) return fail(TG3_ERR_ARG, "null count");
    int cnt = 0;
    TG3_CUDA(cudaGetDeviceCount(&cnt));
    int k = 0;
    for (int d = 0; d < cnt; d++) {
        cudaDeviceProp p;
        TG3_CUDA(cudaGetDeviceProperties(&p, d));
        if (p.major >= 10) {
            if (gpus && k < cap) gpus[k] = d;
            k++;
        }
    }
    *n = k;
    return TG3_OK;
}

// ================================================================== context
extern "C" int tg3_ctx_create(tg3_ctx** out, int device)
{
    if (!out) return fail(TG3_ERR_ARG, "null output");
    *out = nullptr;
    TG3_CUDA(cudaSetDevice(device));
    tg3_ctx* c = new tg3_ctx();
    c->device = device;
    // a blocking stream: ordered with work the caller queued on the legacy
    // default stream (e.g. copies that produced our inputs)
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamDefault);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_flag, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_flag, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_volTable, sizeof(float4*) * kMaxClasses);
    if (e == cudaSuccess) e = cudaMemset(c->d_volTable, 0, sizeof(float4*) * kMaxClasses);
    if (e != cudaSuccess) {
        int st = cuda_fail(e, "context set-up");
        tg3_ctx_destroy(c);
        return st;
    }
    *out = c;
    return TG3_OK;
}

extern "C" int tg3_ctx_destroy(tg3_ctx* c)
{
    if (!c) return TG3_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    prep_release(c);
    reco_release(c);
    for (auto& v : c->vol) cudaFree(v.blocks);
    for (auto& b : c->ws) cudaFree(b.ptr);
    cudaFree(c->pxMain.iCol);
    cudaFree(c->pxMain.iRow);
    cudaFree(c->pxMain.cellPix);
    for (auto& q : c->pxSlot) {
        cudaFree(q.iCol);
        cudaFree(q.iRow);
        cudaFree(q.cellPix);
    }
    cudaFree(c->ins.acc);
    cudaFree(c->ins.tab);
    for (auto& b : c->bank) {
        cudaFree(b.f32);
        cudaFree(b.hi);
        cudaFree(b.abs2);
        cudaFree(b.abs2q);
        cudaFree(b.quat);
        cudaFree(b.emb);
    }
    if (c->copyStream) {
        cudaStreamSynchronize(c->copyStream);
        cudaStreamDestroy(c->copyStream);
    }
    if (c->copyDone) cudaEventDestroy(c->copyDone);
    cudaFree(c->d_bankTable);
    cudaFree(c->d_refTable);
    cudaFree(c->d_flag);
    cudaFree(c->d_volTable);
    for (auto& v : c->pending)
        for (auto& pr : v) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    for (auto e : c->eventPool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TG3_OK;
}

extern "C" void* tg3_ctx_stream(tg3_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int tg3_ctx_sync(tg3_ctx* c)
{
    int st = check_ctx(c);
    if (st) return st;
    return sync_and_check(c);
}

extern "C" size_t tg3_ctx_workspace_bytes(tg3_ctx* c)
{
    if (!c) return 0;
    size_t s = 0;
    for (auto& b : c->ws) s += b.bytes;
    return s;
}

extern "C" int tg3_ctx_set_volume(tg3_ctx* c, int cls, const float* volume, int vdim, int pf,
                                  int on_device)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses) return fail(TG3_ERR_ARG, "class index out of range");
    if (!volume || vdim < 4 || (vdim & 1) || pf < 1) return fail(TG3_ERR_ARG, "bad volume");
    Volume& v = c->vol[cls];
    const size_t nvox = (size_t)vdim * vdim * (vdim / 2 + 1);
    if (volume_block_count(vdim) > (size_t)0x7fffffff)
        return fail(TG3_ERR_ARG, "volume edge too large for 32-bit block indices");
    const size_t bytes = volume_block_count(vdim) * 4 * sizeof(float4);   // 64-byte blocks
    if (v.bytes != bytes) {
        TG3_CUDA(cudaStreamSynchronize(c->stream));
        cudaFree(v.blocks);
        v.blocks = nullptr;
        v.bytes = 0;
        TG3_CUDA(cudaMalloc(&v.blocks, bytes));
        v.bytes = bytes;
    }
    v.vdim = vdim;
    v.pf = pf;
    const float2* src = reinterpret_cast<const float2*>(volume);
    if (!on_device) {
        float2* tmp = nullptr;
        st = upload(c, WS_PAIRS_TMP, 0, src, nvox, &tmp);
        if (st) return st;
        src = tmp;
    }
    TG3_CUDA(launch_volume_blocks(src, vdim, v.blocks, c->stream));
    float4* table[kMaxClasses];
    for (int i = 0; i < kMaxClasses; i++) table[i] = c->vol[i].blocks;
    TG3_CUDA(cudaMemcpyAsync(c->d_volTable, table, sizeof(table), cudaMemcpyHostToDevice,
                             c->stream));
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    return TG3_OK;
}

// Upload a pixel list into an owned set (device buffers grown as needed).
static int upload_pixels(tg3_ctx* c, Pixels& px, const int* iCol, const int* iRow, int K, int idim)
{
    if (!iCol || !iRow || K <= 0 || idim <= 0) return fail(TG3_ERR_ARG, "bad pixel list");
    double mr = 0;
    int ma = 0;
    for (int p = 0; p < K; p++) {
        if (iCol[p] < 0 || std::abs(iCol[p]) > idim / 2 || std::abs(iRow[p]) > idim / 2)
            return fail(TG3_ERR_ARG, "pixel outside the half plane of the image");
        mr = std::max(mr, std::sqrt((double)iCol[p] * iCol[p] + (double)iRow[p] * iRow[p]));
        ma = std::max(ma, std::max(iCol[p], std::abs(iRow[p])));
    }
    // the insertion gather's cell map; a pixel listed twice cannot share a cell
    const size_t cells = (size_t)(ma + 1) * (2 * ma + 1);
    std::vector<int> cell(cells, -1);
    bool unique = true;
    for (int p = 0; p < K && unique; p++) {
        int& s = cell[(size_t)(iRow[p] + ma) * (ma + 1) + iCol[p]];
        unique = s < 0;
        s = p;
    }
    if (px.K != K) {
        TG3_CUDA(cudaStreamSynchronize(c->stream));
        cudaFree(px.iCol);
        cudaFree(px.iRow);
        px.iCol = px.iRow = nullptr;
        px.K = 0;
        TG3_CUDA(cudaMalloc(&px.iCol, sizeof(int) * K));
        TG3_CUDA(cudaMalloc(&px.iRow, sizeof(int) * K));
    }
    TG3_CUDA(cudaMemcpyAsync(px.iCol, iCol, sizeof(int) * K, cudaMemcpyHostToDevice, c->stream));
    TG3_CUDA(cudaMemcpyAsync(px.iRow, iRow, sizeof(int) * K, cudaMemcpyHostToDevice, c->stream));
    if (unique) {
        if (px.cells != cells) {
            TG3_CUDA(cudaStreamSynchronize(c->stream));
            cudaFree(px.cellPix);
            px.cellPix = nullptr;
            px.cells = 0;
            TG3_CUDA(cudaMalloc(&px.cellPix, sizeof(int) * cells));
            px.cells = cells;
        }
        TG3_CUDA(cudaMemcpyAsync(px.cellPix, cell.data(), sizeof(int) * cells,
                                 cudaMemcpyHostToDevice, c->stream));
    }
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    px.K = K;
    px.Kp = (int)round_up(2 * (size_t)K, 64);
    px.idim = idim;
    px.maxRadius = mr;
    px.maxAbs = ma;
    px.unique = unique;
    px.gen = ++c->pixGen;
    return TG3_OK;
}

extern "C" int tg3_ctx_set_pixels(tg3_ctx* c, const int* iCol, const int* iRow, int K,
                                  int idim)
{
    int st = check_ctx(c);
    if (st) return st;
    if ((st = upload_pixels(c, c->pxMain, iCol, iRow, K, idim))) return st;
    c->px = c->pxMain;
    return TG3_OK;
}

extern "C" int tg3_ctx_set_pixels_slot(tg3_ctx* c, int slot, const int* iCol, const int* iRow,
                                       int K, int idim)
{
    int st = check_ctx(c);
    if (st) return st;
    if (slot < 0 || slot >= kMaxClasses) return fail(TG3_ERR_ARG, "pixel slot out of range");
    return upload_pixels(c, c->pxSlot[slot], iCol, iRow, K, idim);
}

extern "C" int tg3_ctx_use_pixels(tg3_ctx* c, int slot)
{
    int st = check_ctx(c);
    if (st) return st;
    if (slot < -1 || slot >= kMaxClasses) return fail(TG3_ERR_ARG, "pixel slot out of range");
    const Pixels& src = slot < 0 ? c->pxMain : c->pxSlot[slot];
    if (!src.iCol) return fail(TG3_ERR_STATE, "pixel set not uploaded");
    c->px = src;
    return TG3_OK;
}

// ======================================================= batched local phase
// Sequence per batch: project (+ per-row norm) -> shifted data bank -> cross
// term GEMM (FP32 CUDA cores or split-bf16 tensor cores) with the norm folded
// into its epilogue -> marginal weights.
static int local_phase(tg3_ctx* c, const int* bankIdx, int nP, int nR, int nT, const float* dat,
                       const float* ctf, const float* sigRcp, const double* quat,
                       const double* trans, const double* pwR, const double* pwT,
                       const double* pwC, const int* cls, double* wC, double* wR,
                       double* wT, double* baseL, float* dvp, int precision)
{
    const int K = c->px.K, Kp = c->px.Kp;
    int st = TG3_OK;
    // volume of every class used must be set; check class 0 geometry
    const Volume& v0 = c->vol[0];
    if (!v0.blocks) return fail(TG3_ERR_STATE, "volume of class 0 not set");
    for (int k = 1; k < kMaxClasses; k++)
        if (c->vol[k].blocks && (c->vol[k].vdim != v0.vdim || c->vol[k].pf != v0.pf))
            return fail(TG3_ERR_ARG, "all class volumes must share one edge and pf");
    if ((st = check_geometry(c, v0.vdim, v0.pf))) return st;
    if ((st = check_weights_shape(nR, nT))) return st;
    const bool fusedPath = precision == TG3_SCORE_BF16X3 && c->fused && !bankIdx;
    float* P = fusedPath ? nullptr
                         : (float*)ws_get(c, WS_P, sizeof(float) * (size_t)nP * nR * Kp, &st);
    if (!fusedPath && !P) return st;
    float* A = (float*)ws_get(c, WS_A, sizeof(float) * (size_t)nP * nT * Kp, &st);
    if (!A) return st;
    float* D = (float*)ws_get(c, WS_D, sizeof(float) * (size_t)nP * nR * nT, &st);
    if (!D) return st;
    float* nrm = (float*)ws_get(c, WS_NRM, sizeof(float) * (size_t)nP * nR, &st);
    if (!nrm) return st;
    float* pscr = (float*)ws_get(
        c, WS_PROJ, sizeof(float) * project_scratch_floats(nP * nR, (int)Kp), &st);
    if (!pscr) return st;
    double* x0 = (double*)ws_get(c, WS_X0, sizeof(double) * (size_t)nP, &st);
    if (!x0) return st;
    cudaStream_t s = c->stream;
    if (precision != TG3_SCORE_FP32 && precision != TG3_SCORE_BF16X3)
        return fail(TG3_ERR_ARG, "unknown precision");
    const bool split = precision == TG3_SCORE_BF16X3;
    if (split && !bf16x3_available())
        return fail(TG3_ERR_UNSUPPORTED, "split-bf16 tensor-core path unavailable (no TMA encoder)");
    if (split && nT > 256) return fail(TG3_ERR_UNSUPPORTED, "split-bf16 path needs nT <= 256");
    // split-bf16: the same buffers hold a hi plane followed by a lo plane
    const long long splitP = split ? (long long)nP * nR * Kp : 0;
    const long long splitA = split ? (long long)nP * nT * Kp : 0;
    if (fusedPath) {
        // projection + cross term in one kernel; the slices stay on chip
        const size_t partBytes = round_up(sizeof(FusedParticle) * (size_t)nP, 256);
        const size_t offBytes = round_up(sizeof(int) * ((size_t)nP + 1), 256);
        char* fw = (char*)ws_get(c, WS_FUSED, partBytes + offBytes + 256, &st);
        if (!fw) return st;
        FusedParticle* part = reinterpret_cast<FusedParticle*>(fw);
        int* itemOff = reinterpret_cast<int*>(fw + partBytes);
        int* counter = reinterpret_cast<int*>(fw + partBytes + offBytes);
        {
            StageTimer tm(c, TG3_STAGE_SHIFT);
            TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(dat), ctf, sigRcp, trans,
                                       nullptr, nP, nT, c->px.idim, c->px.iCol, c->px.iRow, K, A,
                                       Kp, splitA, s));
            TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(dat), sigRcp, nP, K, x0, s));
            TG3_CUDA(launch_rot_f32(quat, nullptr, nP * nR, pscr, s));
            TG3_CUDA(launch_fused_uniform_setup(nP, nR, nT, K, cls, part, itemOff, s));
        }
        {
            StageTimer tm(c, TG3_STAGE_FUSED);
            FusedPixels pix[kMaxClasses];
            for (int k = 0; k < kMaxClasses; k++) pix[k] = {c->px.iCol, c->px.iRow, K, Kp};
            TG3_CUDA(launch_fused_bf16x3(c->d_volTable, v0.vdim, v0.pf, pscr, part, itemOff, nP,
                                         nP * fused_items(nR), pix, sigRcp, ctf, A,
                                         (long long)nP * nT, Kp, nT, D, -2.0f, c->d_flag,
                                         counter, s));
        }
        {
            StageTimer tm(c, TG3_STAGE_WEIGHTS);
            TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, nP, nullptr, 0, x0, pwR,
                                    nR, pwT, nT, pwC, wC, wR, wT, baseL, dvp, s));
        }
        return TG3_OK;
    }
    if (bankIdx && split && c->bankGather != 1) {
        // the cross term reads the proposed rows straight from the banks and
        // sums their norms itself: no slice copy, no |P|^2 rows
        {
            StageTimer tm(c, TG3_STAGE_SHIFT);
            TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(dat), ctf, sigRcp, trans,
                                       nullptr, nP, nT, c->px.idim, c->px.iCol, c->px.iRow, K,
                                       A, Kp, splitA, s));
            TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(dat), sigRcp, nP, K, x0, s));
        }
        {
            StageTimer tm(c, TG3_STAGE_CROSS);
            int* order = nullptr;
            if (c->bankOrder && nP <= 8192) {
                int ost = TG3_OK;
                order = (int*)ws_get(c, WS_ORDER, sizeof(int) * (size_t)nP, &ost);
                if (!order) return ost;
            }
            TG3_CUDA(launch_gemm_bank_bf16x3(c->bank, c->px.gen, bankIdx, cls, nP, nR, A, nT, Kp,
                                             K, sigRcp, ctf, D, -2.0f, c->d_flag, s,
                                             c->bankGather == 2, order, c->bankShape));
        }
        {
            StageTimer tm(c, TG3_STAGE_WEIGHTS);
            TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, nP, nullptr, 0, x0, pwR,
                                    nR, pwT, nT, pwC, wC, wR, wT, baseL, dvp, s));
        }
        return TG3_OK;
    }
    if (bankIdx) {
        StageTimer tm(c, TG3_STAGE_PROJECT);
        TG3_CUDA(launch_bank_gather(c->d_bankTable, cls, bankIdx, nP, nR, K, Kp, sigRcp, ctf, P,
                                    splitP, nrm, c->d_flag, s));
    } else {
        StageTimer tm(c, TG3_STAGE_PROJECT);
        TG3_CUDA(launch_project(c->d_volTable, cls, nullptr, v0.vdim, v0.pf, quat, nullptr,
                                nP * nR, nR, c->px.iCol, c->px.iRow, K, P, Kp, sigRcp, ctf, nrm,
                                pscr, c->d_flag, splitP, s, c->projForm, c->projGroup));
    }
    {
        StageTimer tm(c, TG3_STAGE_SHIFT);
        TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(dat), ctf, sigRcp, trans,
                                   nullptr, nP, nT, c->px.idim, c->px.iCol, c->px.iRow, K, A, Kp,
                                   splitA, s));
        TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(dat), sigRcp, nP, K, x0, s));
    }
    {
        StageTimer tm(c, TG3_STAGE_CROSS);
        if (split)
            TG3_CUDA(launch_gemm_nt_bf16x3(P, (long long)nR * Kp, Kp, A, (long long)nT * Kp, Kp,
                                           nR, nT, Kp, nP, D, (long long)nR * nT, nT, nrm, nR,
                                           -2.0f, nullptr, 0, c->d_flag, s, c->localBK));
        else
            TG3_CUDA(launch_gemm_nt_fp32(P, (long long)nR * Kp, Kp, A, (long long)nT * Kp, Kp, nR,
                                         nT, Kp, nP, D, (long long)nR * nT, nT, nrm, nR, -2.0f,
                                         s));
    }
    {
        StageTimer tm(c, TG3_STAGE_WEIGHTS);
        TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, nP, nullptr, 0, x0, pwR, nR,
                                pwT, nT, pwC, wC, wR, wT, baseL, dvp, s));
    }
    return TG3_OK;
}

extern "C" int tg3_local_phase_d(tg3_ctx* c, int nP, int nR, int nT, const float* dat,
                                 const float* ctf, const float* sigRcp, const double* quat,
                                 const double* trans, const double* pwR, const double* pwT,
                                 const double* pwC, const int* cls, double* wC, double* wR,
                                 double* wT, double* baseL, float* dvp, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (nP <= 0 || nR <= 0 || nT <= 0 || nT > 2048) return fail(TG3_ERR_ARG, "bad batch shape (nT <= 2048)");
    if (!dat || !ctf || !sigRcp || !quat || !trans || !pwR || !pwT || !wC || !wR || !wT || !baseL)
        return fail(TG3_ERR_ARG, "null device pointer");
    return local_phase(c, nullptr, nP, nR, nT, dat, ctf, sigRcp, quat, trans, pwR, pwT, pwC, cls, wC, wR,
                       wT, baseL, dvp, precision);
}

// ========================================================== defocus search
// The local phase with a defocus axis (Optimiser::updateSP,
// src/Optimiser.cpp:1139-1436, SEARCH_TYPE_CTF): every (rotation,
// translation, defocus) hypothesis scored with the particle's CTF for that
// defocus.  The weights kernel takes (particle, defocus) blocks, each with
// its own maximum; k_merge_defocus rescales them to the particle's maximum.
static int local_phase_ctf(tg3_ctx* c, int nP, int nR, int nT, int nD, const float* dat,
                           const float* ctfD, const float* sigRcp, const double* quat,
                           const double* trans, const double* pwR, const double* pwT,
                           const double* pwD, const double* pwC, const int* cls, double* wC,
                           double* wR, double* wT, double* wD, double* baseL, float* dvp,
                           int precision)
{
    int st = TG3_OK;
    if (nP <= 0 || nR <= 0 || nT <= 0 || nD < 1 || nD > 16)
        return fail(TG3_ERR_ARG, "bad batch shape (1 <= nD <= 16)");
    if (!dat || !ctfD || !sigRcp || !quat || !trans || !pwR || !pwT || !pwD || !wC || !wR ||
        !wT || !wD || !baseL)
        return fail(TG3_ERR_ARG, "null device pointer");
    if (precision != TG3_SCORE_FP32 && precision != TG3_SCORE_BF16X3)
        return fail(TG3_ERR_ARG, "unknown precision");
    const bool split = precision == TG3_SCORE_BF16X3;
    if (split && !bf16x3_available())
        return fail(TG3_ERR_UNSUPPORTED, "split-bf16 tensor-core path unavailable (no TMA encoder)");
    if (split && nD * nT > 256)
        return fail(TG3_ERR_UNSUPPORTED, "split-bf16 path needs nD nT <= 256");
    const int K = c->px.K, Kp = c->px.Kp;
    const Volume& v0 = c->vol[0];
    if (!v0.blocks) return fail(TG3_ERR_STATE, "volume of class 0 not set");
    if ((st = check_geometry(c, v0.vdim, v0.pf))) return st;
    if ((st = check_weights_shape(nR, nT))) return st;
    const int nTD = nD * nT;
    float* P = (float*)ws_get(c, WS_P, sizeof(float) * (size_t)nP * nR * Kp, &st);
    if (!P) return st;
    float* A = (float*)ws_get(c, WS_A, sizeof(float) * (size_t)nP * nTD * Kp, &st);
    if (!A) return st;
    float* D = (float*)ws_get(c, WS_D, sizeof(float) * (size_t)nP * nR * nTD, &st);
    if (!D) return st;
    float* nrm = (float*)ws_get(c, WS_NRM, sizeof(float) * (size_t)nP * nR * nD, &st);
    if (!nrm) return st;
    float* pscr = (float*)ws_get(
        c, WS_PROJ, sizeof(float) * project_scratch_floats(nP * nR, (int)Kp), &st);
    if (!pscr) return st;
    double* x0 = (double*)ws_get(c, WS_X0, sizeof(double) * (size_t)nP, &st);
    if (!x0) return st;
    // per-block priors, x0 and weights: blocks (l, d)
    const size_t nB = (size_t)nP * nD;
    const size_t dbl = nB * ((size_t)nR + nT + 2) * 2 + 2 * nB;
    double* dw = (double*)ws_get(c, WS_DEFOCUS, sizeof(double) * dbl, &st);
    if (!dw) return st;
    double* pRb = dw;
    double* pTb = pRb + nB * nR;
    double* pCb = pTb + nB * nT;
    double* x0b = pCb + nB;
    double* wRb = x0b + nB;
    double* wTb = wRb + nB * nR;
    double* wCb = wTb + nB * nT;
    double* bb = wCb + nB;
    cudaStream_t s = c->stream;
    const long long splitP = split ? (long long)nP * nR * Kp : 0;
    const long long splitA = split ? (long long)nP * nTD * Kp : 0;
    {
        StageTimer tm(c, TG3_STAGE_PROJECT);
        TG3_CUDA(launch_project(c->d_volTable, cls, nullptr, v0.vdim, v0.pf, quat, nullptr,
                                nP * nR, nR, c->px.iCol, c->px.iRow, K, P, Kp, nullptr, nullptr,
                                nullptr, pscr, c->d_flag, splitP, s, c->projForm, c->projGroup));
        TG3_CUDA(launch_norm_defocus(P, splitP, nP, nR, nD, K, Kp, sigRcp, ctfD, nrm, s));
    }
    {
        StageTimer tm(c, TG3_STAGE_SHIFT);
        TG3_CUDA(launch_shift_bank(reinterpret_cast<const float2*>(dat), ctfD, sigRcp, trans,
                                   nullptr, nP, nT, c->px.idim, c->px.iCol, c->px.iRow, K, A, Kp,
                                   splitA, s, nD));
        TG3_CUDA(launch_x0(reinterpret_cast<const float2*>(dat), sigRcp, nP, K, x0, s));
    }
    {
        StageTimer tm(c, TG3_STAGE_CROSS);
        if (split)
            TG3_CUDA(launch_gemm_nt_bf16x3(P, (long long)nR * Kp, Kp, A, (long long)nTD * Kp, Kp,
                                           nR, nTD, Kp, nP, D, (long long)nR * nTD, nTD, nullptr,
                                           nR, -2.0f, nullptr, 0, c->d_flag, s));
        else
            TG3_CUDA(launch_gemm_nt_fp32(P, (long long)nR * Kp, Kp, A, (long long)nTD * Kp, Kp,
                                         nR, nTD, Kp, nP, D, (long long)nR * nTD, nTD, nullptr,
                                         nR, -2.0f, s));
    }
    {
        StageTimer tm(c, TG3_STAGE_WEIGHTS);
        TG3_CUDA(launch_repeat_rows(pwR, nP, nR, nD, pRb, s));
        TG3_CUDA(launch_repeat_rows(pwT, nP, nT, nD, pTb, s));
        TG3_CUDA(launch_repeat_rows(pwC, nP, 1, nD, pCb, s));
        TG3_CUDA(launch_repeat_rows(x0, nP, 1, nD, x0b, s));
        TG3_CUDA(launch_weights(D, (long long)nR * nTD, nTD, nR, nT, nD, (int)nB, nrm,
                                (int)nB, x0b, pRb, nR, pTb, nT, pCb, wCb, wRb, wTb, bb, dvp, s));
        TG3_CUDA(launch_merge_defocus(nP, nD, nR, nT, wCb, wRb, wTb, bb, pwD, wC, wR, wT, wD,
                                      baseL, s));
    }
    return TG3_OK;
}

extern "C" int tg3_local_phase_ctf_d(tg3_ctx* c, int nP, int nR, int nT, int nD,
                                     const float* dat, const float* ctfD, const float* sigRcp,
                                     const double* quat, const double* trans, const double* pwR,
                                     const double* pwT, const double* pwD, const double* pwC,
                                     const int* cls, double* wC, double* wR, double* wT,
                                     double* wD, double* baseL, float* dvp, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    return local_phase_ctf(c, nP, nR, nT, nD, dat, ctfD, sigRcp, quat, trans, pwR, pwT, pwD, pwC,
                           cls, wC, wR, wT, wD, baseL, dvp, precision);
}

// ================================================================= banks
// Upload the device views of the banks and of the references; a bank built
// on another pixel set than the active one shows no rows, so an index into
// it is flagged, and its references are not offered.
int tg3::upload_bank_views(tg3_ctx* c, bool* anyBank, bool* anyRef)
{
    if (!c->d_bankTable) TG3_CUDA(cudaMalloc(&c->d_bankTable, sizeof(BankView) * kMaxClasses));
    if (!c->d_refTable) TG3_CUDA(cudaMalloc(&c->d_refTable, sizeof(RefView) * kMaxClasses));
    BankView view[kMaxClasses];
    RefView ref[kMaxClasses];
    bool any = false, anyR = false;
    for (int k = 0; k < kMaxClasses; k++) {
        const Bank& q = c->bank[k];
        const bool ok = q.nB > 0 && q.gen == c->px.gen && q.K == c->px.K;
        const size_t rf = (size_t)q.nB * q.Kp;
        view[k] = {q.f32, q.hi, q.hi ? q.hi + rf : nullptr, q.abs2, ok ? q.nB : 0};
        const bool okR = ok && q.emb && q.nEmb == q.nB;
        ref[k] = {q.emb, q.quat, okR ? q.nEmb : 0};
        any = any || ok;
        anyR = anyR || okR;
    }
    TG3_CUDA(cudaMemcpyAsync(c->d_bankTable, view, sizeof(view), cudaMemcpyHostToDevice,
                             c->stream));
    TG3_CUDA(cudaMemcpyAsync(c->d_refTable, ref, sizeof(ref), cudaMemcpyHostToDevice,
                             c->stream));
    if (anyBank) *anyBank = any;
    if (anyRef) *anyRef = anyR;
    // (copies from pageable memory return once the source has been staged)
    return TG3_OK;
}

static int upload_bank_table(tg3_ctx* c, bool* anyValid)
{
    return upload_bank_views(c, anyValid, nullptr);
}

extern "C" int tg3_ctx_set_bank(tg3_ctx* c, int cls, const double* quat, int nB)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks)
        return fail(TG3_ERR_STATE, "volume of the bank's class not set");
    if (!quat || nB <= 0) return fail(TG3_ERR_ARG, "bad bank arguments");
    const Volume& v = c->vol[cls];
    if ((st = check_geometry(c, v.vdim, v.pf))) return st;
    const int K = c->px.K, Kp = c->px.Kp;
    Bank& b = c->bank[cls];
    const size_t rowF = (size_t)nB * Kp;
    const size_t need = rowF * sizeof(float) + 2 * rowF * sizeof(__nv_bfloat16) +
                        (size_t)nB * K * sizeof(float);
    // the references and the |P|^2 rows belong to the previous rotation set
    b.nEmb = 0;
    b.abs2qSplit = -1;
    if (b.bytes < need || b.nB != nB) {
        TG3_CUDA(cudaStreamSynchronize(c->stream));
        cudaFree(b.f32);
        cudaFree(b.hi);
        cudaFree(b.abs2);
        cudaFree(b.abs2q);
        cudaFree(b.quat);
        cudaFree(b.emb);
        b = Bank();
        TG3_CUDA(cudaMalloc(&b.quat, (size_t)nB * 4 * sizeof(double)));
        TG3_CUDA(cudaMalloc(&b.f32, rowF * sizeof(float)));
        TG3_CUDA(cudaMalloc(&b.hi, 2 * rowF * sizeof(__nv_bfloat16)));
        TG3_CUDA(cudaMalloc(&b.abs2, (size_t)nB * K * sizeof(float)));
        b.bytes = need;
    }
    float* pscr = (float*)ws_get(c, WS_PROJ, sizeof(float) * project_scratch_floats(nB, Kp), &st);
    if (!pscr) return st;
    TG3_CUDA(launch_project(nullptr, nullptr, v.blocks, v.vdim, v.pf, quat, nullptr, nB, nB,
                            c->px.iCol, c->px.iRow, K, b.f32, Kp, nullptr, nullptr, nullptr, pscr,
                            c->d_flag, 0, c->stream, c->projForm, c->projGroup));
    TG3_CUDA(launch_bank_planes(b.f32, nB, K, Kp, b.hi, b.hi + rowF, b.abs2, c->stream));
    TG3_CUDA(cudaMemcpyAsync(b.quat, quat, (size_t)nB * 4 * sizeof(double),
                             cudaMemcpyDeviceToDevice, c->stream));
    b.nB = nB;
    b.K = K;
    b.Kp = Kp;
    b.gen = c->px.gen;
    if ((st = upload_bank_table(c, nullptr))) return st;
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    return TG3_OK;
}

extern "C" int tg3_local_phase_bank_d(tg3_ctx* c, int nP, int nR, int nT, const float* dat,
                                      const float* ctf, const float* sigRcp, const int* bankIdx,
                                      const double* trans, const double* pwR, const double* pwT,
                                      const double* pwC, const int* cls, double* wC, double* wR,
                                      double* wT, double* baseL, float* dvp, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (nP <= 0 || nR <= 0 || nT <= 0 || nT > 2048) return fail(TG3_ERR_ARG, "bad batch shape (nT <= 2048)");
    if (!dat || !ctf || !sigRcp || !bankIdx || !trans || !pwR || !pwT || !wC || !wR || !wT ||
        !baseL)
        return fail(TG3_ERR_ARG, "null device pointer");
    // the classes are device data: banks built on another pixel set show no
    // rows, and a particle that names one is flagged
    bool any = false;
    if ((st = upload_bank_table(c, &any))) return st;
    if (!any) return fail(TG3_ERR_STATE, "no projection bank built on the active pixel set");
    return local_phase(c, bankIdx, nP, nR, nT, dat, ctf, sigRcp, nullptr, trans, pwR, pwT, pwC,
                       cls, wC, wR, wT, baseL, dvp, precision);
}

// ================================================================ resample
extern "C" int tg3_resample_d(tg3_ctx* c, int nP, int n, const double* u, const double* w,
                              const int* perm, const double* u0, const double* peak, int nOut,
                              int* src, double* wOut, int* top)
{
    int st = check_ctx(c);
    if (st) return st;
    if (nP <= 0 || n <= 0 || nOut <= 0 || n > kMaxResampleN || nOut > kMaxResampleN)
        return fail(TG3_ERR_ARG, "resample sizes out of range (1.." +
                                     std::to_string(kMaxResampleN) + ")");
    if (!u || !w || !perm || !u0 || !src || !wOut || !top) return fail(TG3_ERR_ARG, "null pointer");
    StageTimer tm(c, TG3_STAGE_RESAMPLE);
    TG3_CUDA(launch_resample(nP, n, u, w, perm, u0, peak, nOut, src, wOut, top, c->d_flag,
                             c->stream));
    return TG3_OK;
}

extern "C" int tg3_resample(int nP, int n, const double* u, const double* w, const int* perm,
                            const double* u0, const double* peak, int nOut, int* src,
                            double* wOut, int* top)
{
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    if (nP <= 0 || n <= 0 || nOut <= 0) return fail(TG3_ERR_ARG, "bad sizes");
    if (!u || !w || !perm || !u0 || !src || !wOut || !top) return fail(TG3_ERR_ARG, "null pointer");
    Arena ar(c, WS_H2D);
    const size_t nn = (size_t)nP * n, no = (size_t)nP * nOut;
    size_t ou = ar.add(nn * 8), ow = ar.add(nn * 8), op = ar.add(nn * 4), o0 = ar.add(nP * 8),
           opk = ar.add(nP * 8), os = ar.add(no * 4), owo = ar.add(no * 8), ot = ar.add(nP * 4);
    char* base = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!base) return st;
    cudaStream_t s = c->stream;
    TG3_CUDA(cudaMemcpyAsync(base + ou, u, nn * 8, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(base + ow, w, nn * 8, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(base + op, perm, nn * 4, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(base + o0, u0, nP * 8, cudaMemcpyHostToDevice, s));
    if (peak) TG3_CUDA(cudaMemcpyAsync(base + opk, peak, nP * 8, cudaMemcpyHostToDevice, s));
    st = tg3_resample_d(c, nP, n, (double*)(base + ou), (double*)(base + ow), (int*)(base + op),
                        (double*)(base + o0), peak ? (double*)(base + opk) : nullptr, nOut,
                        (int*)(base + os), (double*)(base + owo), (int*)(base + ot));
    if (st) return st;
    if ((st = sync_and_check(c))) return st;
    TG3_CUDA(cudaMemcpy(src, base + os, no * 4, cudaMemcpyDeviceToHost));
    TG3_CUDA(cudaMemcpy(wOut, base + owo, no * 8, cudaMemcpyDeviceToHost));
    TG3_CUDA(cudaMemcpy(top, base + ot, nP * 4, cudaMemcpyDeviceToHost));
    return TG3_OK;
}

// =============================================================== insertion
extern "C" int tg3_ctx_insert_begin(tg3_ctx* c, int vdim, int pf)
{
    int st = check_ctx(c);
    if (st) return st;
    if (vdim < 4 || (vdim & 1) || pf < 1) return fail(TG3_ERR_ARG, "bad insertion volume");
    InsertAcc& in = c->ins;
    const size_t bytes = (size_t)vdim * vdim * (vdim / 2 + 1) * sizeof(float4);
    if (in.bytes != bytes) {
        TG3_CUDA(cudaStreamSynchronize(c->stream));
        cudaFree(in.acc);
        in.acc = nullptr;
        in.bytes = 0;
        TG3_CUDA(cudaMalloc(&in.acc, bytes));
        in.bytes = bytes;
    }
    if (in.pf != pf || !in.tab) {
        std::vector<float> tab;
        int nz = 0;
        const double b = (pf * kMkbA) * (pf * kMkbA);
        mkb_table(kMkbA, kMkbAlpha, b, kMkbN, tab, nz);
        TG3_CUDA(cudaStreamSynchronize(c->stream));
        cudaFree(in.tab);
        in.tab = nullptr;
        TG3_CUDA(cudaMalloc(&in.tab, sizeof(float) * (nz + 1)));
        TG3_CUDA(cudaMemcpy(in.tab, tab.data(), sizeof(float) * (nz + 1), cudaMemcpyHostToDevice));
        in.tabNz = nz;
        in.tabInvStep = (float)(kMkbN / b);
    }
    in.vdim = vdim;
    in.pf = pf;
    TG3_CUDA(cudaMemsetAsync(in.acc, 0, bytes, c->stream));
    return TG3_OK;
}

// ctfRows == nDraws: one CTF row per draw (the defocus search), else one
// per image
// nC (device, per image; NULL: every draw): draw m of image l is inserted
// only when m < nC[l] (the multi-class InsertFT); it takes the scatter form.
static int insert_draws(tg3_ctx* c, int nDraws, int drawsPerImage, const float* dat,
                        const float* ctf, const double* quat, const double* trans,
                        const double* offset, const float* w, int kernel, double* O3D,
                        int* counter, int ctfRows = 0, const int* nC = nullptr)
{
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "insertion volume not begun");
    if (kernel != TG3_KERNEL_MKB && kernel != TG3_KERNEL_TRILINEAR)
        return fail(TG3_ERR_ARG, "unknown insertion kernel");
    int st = check_geometry(c, c->ins.vdim, c->ins.pf, 2.0);
    if (st) return st;
    StageTimer tm(c, TG3_STAGE_INSERT);
    if (kernel == TG3_KERNEL_MKB && c->insertGather && c->px.unique && c->px.cellPix && !nC) {
        const size_t per = insert_draw_bytes(c->px.maxAbs);
        const size_t bytes = std::max(per, std::min((size_t)nDraws * per, (size_t)96 << 20));
        void* scratch = ws_get(c, WS_INSERT, bytes, &st);
        if (st) return st;
        TG3_CUDA(launch_insert_gather(c->ins.acc, c->ins.vdim, c->ins.tab, c->ins.tabNz,
                                      c->ins.tabInvStep, nDraws, drawsPerImage,
                                      reinterpret_cast<const float2*>(dat), ctf, quat, trans,
                                      offset, w, c->px.cellPix, c->px.iCol, c->px.iRow,
                                      c->px.K, c->ins.pf,
                                      c->px.idim, c->px.maxAbs,
                                      (float)(c->px.maxRadius * c->ins.pf), O3D, counter,
                                      scratch, bytes, c->stream, ctfRows));
        return TG3_OK;
    }
    float* params = static_cast<float*>(
        ws_get(c, WS_INSERT, (size_t)nDraws * 16 * sizeof(float), &st));
    if (st) return st;
    TG3_CUDA(launch_insert(c->ins.acc, c->ins.vdim, kernel, c->ins.tab, c->ins.tabNz,
                           c->ins.tabInvStep, nDraws, drawsPerImage,
                           reinterpret_cast<const float2*>(dat), ctf, quat, trans, offset, w,
                           c->px.iCol, c->px.iRow, c->px.K, c->ins.pf, c->px.idim, O3D,
                           counter, params, c->stream, ctfRows, nC));
    return TG3_OK;
}

extern "C" int tg3_insert_d(tg3_ctx* c, int nP, const float* dat, const float* ctf,
                            const double* quat, const double* trans, const double* offset,
                            const float* w, int kernel, double* O3D, int* counter)
{
    int st = check_ctx(c);
    if (st) return st;
    if (nP <= 0 || !dat || !ctf || !quat || !trans || !w) return fail(TG3_ERR_ARG, "bad insert args");
    return insert_draws(c, nP, 1, dat, ctf, quat, trans, offset, w, kernel, O3D, counter);
}

extern "C" int tg3_ctx_insert_read_d(tg3_ctx* c, float* F, float* T, int accumulate)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "insertion volume not begun");
    if (!F || !T) return fail(TG3_ERR_ARG, "null output");
    const size_t n = (size_t)c->ins.vdim * c->ins.vdim * (c->ins.vdim / 2 + 1);
    TG3_CUDA(launch_acc_read(c->ins.acc, n, reinterpret_cast<float2*>(F), T, accumulate,
                             c->stream));
    return TG3_OK;
}

extern "C" int tg3_ctx_insert_ratio_d(tg3_ctx* c, float* V, float floor_)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!c->ins.acc) return fail(TG3_ERR_STATE, "insertion volume not begun");
    if (!V || !(floor_ >= 0.f)) return fail(TG3_ERR_ARG, "bad ratio args");
    const size_t n = (size_t)c->ins.vdim * c->ins.vdim * (c->ins.vdim / 2 + 1);
    TG3_CUDA(launch_acc_ratio(c->ins.acc, n, floor_, reinterpret_cast<float2*>(V), c->stream));
    return TG3_OK;
}

extern "C" int tg3_fsc_d(const float* A, const float* B, int vdim, int nShell, double* fsc,
                         double* scratch, void* stream)
{
    if (!A || !B || !fsc || !scratch || vdim < 2 || (vdim & 1) || nShell < 1 ||
        (size_t)nShell * 3 * sizeof(double) > 200 * 1024)
        return fail(TG3_ERR_ARG, "bad fsc args");
    TG3_CUDA(launch_fsc(reinterpret_cast<const float2*>(A), reinterpret_cast<const float2*>(B),
                        vdim, nShell, scratch, fsc, (cudaStream_t)stream));
    return TG3_OK;
}

// ======================================================= kernel-level calls
extern "C" int tg3_rotmat_d(const double* quat, int n, double* mat, void* stream)
{
    if (!quat || !mat || n <= 0) return fail(TG3_ERR_ARG, "bad rotmat args");
    TG3_CUDA(launch_rotmat(quat, n, mat, (cudaStream_t)stream));
    return TG3_OK;
}

extern "C" int tg3_translate_d(const double* trans, int nT, int idim, const int* iCol,
                               const int* iRow, int K, float* out, void* stream)
{
    if (!trans || !iCol || !iRow || !out || nT <= 0 || K <= 0 || idim <= 0)
        return fail(TG3_ERR_ARG, "bad translate args");
    TG3_CUDA(launch_translate(trans, nT, idim, iCol, iRow, K, reinterpret_cast<float2*>(out), K,
                              (cudaStream_t)stream));
    return TG3_OK;
}

extern "C" int tg3_ctf_d(const float* attr, int nImg, float pixelSize, int idim,
                         const int* iCol, const int* iRow, int K, float* out, void* stream)
{
    if (!attr || !iCol || !iRow || !out || nImg <= 0 || K <= 0 || pixelSize <= 0)
        return fail(TG3_ERR_ARG, "bad ctf args");
    TG3_CUDA(launch_ctf(attr, nImg, pixelSize, idim, iCol, iRow, K, out, (cudaStream_t)stream));
    return TG3_OK;
}

extern "C" int tg3_project_d(tg3_ctx* c, int cls, const double* rotMat, int nR, float* out)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks) return fail(TG3_ERR_STATE, "volume not set");
    if (!rotMat || !out || nR <= 0) return fail(TG3_ERR_ARG, "bad project args");
    const Volume& v = c->vol[cls];
    if ((st = check_geometry(c, v.vdim, v.pf))) return st;
    float* pscr = (float*)ws_get(
        c, WS_PROJ, sizeof(float) * project_scratch_floats(nR, 2 * c->px.K), &st);
    if (!pscr) return st;
    TG3_CUDA(launch_project(nullptr, nullptr, v.blocks, v.vdim, v.pf, nullptr, rotMat, nR, nR,
                            c->px.iCol, c->px.iRow, c->px.K, out, 2 * c->px.K, nullptr, nullptr,
                            nullptr, pscr, c->d_flag, 0, c->stream, c->projForm, c->projGroup));
    return TG3_OK;
}

// ============================================ reference-shaped entry points
extern "C" int tg3_ExpectRotran(float* traP, const double* trans, const double* rot,
                                double* rotMat, const int* iCol, const int* iRow, int nR,
                                int nT, int idim, int npxl)
{
    if (!traP || !trans || !rot || !rotMat || !iCol || !iRow || nR <= 0 || nT <= 0 || npxl <= 0 ||
        idim <= 0)
        return fail(TG3_ERR_ARG, "bad ExpectRotran args");
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    Arena ar(c, WS_H2D);
    size_t ot = ar.add(sizeof(double) * 2 * nT), orr = ar.add(sizeof(double) * 4 * nR),
           oc = ar.add(sizeof(int) * npxl), orw = ar.add(sizeof(int) * npxl),
           om = ar.add(sizeof(double) * 9 * nR), otr = ar.add(sizeof(float) * 2 * (size_t)nT * npxl);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    cudaStream_t s = c->stream;
    TG3_CUDA(cudaMemcpyAsync(b + ot, trans, sizeof(double) * 2 * nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + orr, rot, sizeof(double) * 4 * nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oc, iCol, sizeof(int) * npxl, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + orw, iRow, sizeof(int) * npxl, cudaMemcpyHostToDevice, s));
    TG3_CUDA(launch_translate((double*)(b + ot), nT, idim, (int*)(b + oc), (int*)(b + orw), npxl,
                              (float2*)(b + otr), npxl, s));
    TG3_CUDA(launch_rotmat((double*)(b + orr), nR, (double*)(b + om), s));
    TG3_CUDA(cudaMemcpyAsync(traP, b + otr, sizeof(float) * 2 * (size_t)nT * npxl,
                             cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(rotMat, b + om, sizeof(double) * 9 * nR, cudaMemcpyDeviceToHost, s));
    return sync_and_check(c);
}

extern "C" int tg3_ExpectProject(const float* volume, float* rotP, const double* rotMat,
                                 const int* iCol, const int* iRow, int nR, int pf, int interp,
                                 int vdim, int npxl)
{
    if (!volume || !rotP || !rotMat || !iCol || !iRow || nR <= 0 || pf < 1 || vdim < 4 || npxl <= 0)
        return fail(TG3_ERR_ARG, "bad ExpectProject args");
    if (interp != 1) return fail(TG3_ERR_UNSUPPORTED, "only linear interpolation (interp 1)");
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    const int slot = kMaxClasses - 1;   // reserved for the reference-shaped calls
    if ((st = tg3_ctx_set_volume(c, slot, volume, vdim, pf, 0))) return st;
    if ((st = tg3_ctx_set_pixels(c, iCol, iRow, npxl, vdim / pf))) return st;
    Arena ar(c, WS_H2D);
    size_t om = ar.add(sizeof(double) * 9 * nR), oo = ar.add(sizeof(float) * 2 * (size_t)nR * npxl);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    TG3_CUDA(cudaMemcpyAsync(b + om, rotMat, sizeof(double) * 9 * nR, cudaMemcpyHostToDevice,
                             c->stream));
    if ((st = tg3_project_d(c, slot, (double*)(b + om), nR, (float*)(b + oo)))) return st;
    TG3_CUDA(cudaMemcpyAsync(rotP, b + oo, sizeof(float) * 2 * (size_t)nR * npxl,
                             cudaMemcpyDeviceToHost, c->stream));
    return sync_and_check(c);
}

// |P|^2 rows and sigRcp ctf^2 rows for the per-(image, rotation) norm GEMM.
namespace tg3 {
__global__ void k_abs2_rows(const float2* __restrict__ in, int K, int rows, float* __restrict__ out,
                            int ldo)
{
    const int r = blockIdx.y;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldo; p += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (p < K) {
            const float2 a = in[(size_t)r * K + p];
            v = a.x * a.x + a.y * a.y;
        }
        out[(size_t)r * ldo + p] = v;
    }
}
__global__ void k_sc2_rows(const float* __restrict__ sig, const float* __restrict__ ctf, int K,
                           float* __restrict__ out, int ldo)
{
    const int r = blockIdx.y;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldo; p += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (p < K) {
            const float c = ctf[(size_t)r * K + p];
            v = sig[(size_t)r * K + p] * c * c;
        }
        out[(size_t)r * ldo + p] = v;
    }
}
__global__ void k_pad_rows(const float2* __restrict__ in, int K, float2* __restrict__ out, int ldo2)
{
    const int r = blockIdx.y;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldo2; p += gridDim.x * blockDim.x)
        out[(size_t)r * ldo2 + p] = p < K ? in[(size_t)r * K + p] : make_float2(0.f, 0.f);
}
}  // namespace tg3

extern "C" int tg3_ExpectGlobal3D(const float* rotP, const float* traP, const float* datP,
                                  const float* ctfP, const float* sigRcpP, float* wC, float* wR,
                                  float* wT, const double* pR, const double* pT, float* baseL,
                                  int kIdx, int nK, int nR, int nT, int npxl, int imgNum)
{
    if (!rotP || !traP || !datP || !ctfP || !sigRcpP || !wC || !wR || !wT || !pR || !pT || !baseL)
        return fail(TG3_ERR_ARG, "null pointer");
    if (nK <= 0 || kIdx < 0 || kIdx >= nK || nR <= 0 || nT <= 0 || npxl <= 0 || imgNum <= 0 ||
        nT > 4096)
        return fail(TG3_ERR_ARG, "bad ExpectGlobal3D sizes");
    int st = check_weights_shape(nR, nT);
    if (st) return st;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    cudaStream_t s = c->stream;
    const int K = npxl, Kp = (int)round_up(2 * (size_t)K, 64), Kq = (int)round_up(K, 64);
    // rotation bank, padded rows, and its |P|^2
    float* P = (float*)ws_get(c, WS_P, sizeof(float) * ((size_t)nR * Kp + (size_t)nR * Kq), &st);
    if (!P) return st;
    float* P2 = P + (size_t)nR * Kp;
    Arena ar(c, WS_H2D);
    size_t orp = ar.add(sizeof(float) * 2 * (size_t)nR * K), otp = ar.add(sizeof(float) * 2 * (size_t)nT * K),
           opr = ar.add(sizeof(double) * nR), opt = ar.add(sizeof(double) * nT);
    const int IB = 1024;   // images per pass
    const int nb = std::min(imgNum, IB);
    size_t od = ar.add(sizeof(float) * 2 * (size_t)nb * K), oc = ar.add(sizeof(float) * (size_t)nb * K),
           os = ar.add(sizeof(float) * (size_t)nb * K), osc = ar.add(sizeof(float) * (size_t)nb * Kq),
           ox0 = ar.add(sizeof(double) * nb), owc = ar.add(sizeof(double) * nb),
           owr = ar.add(sizeof(double) * (size_t)nb * nR), owt = ar.add(sizeof(double) * (size_t)nb * nT),
           obs = ar.add(sizeof(double) * nb), onr = ar.add(sizeof(float) * (size_t)nR * nb),
           oWC = ar.add(sizeof(float) * (size_t)nb * nK), oWR = ar.add(sizeof(float) * (size_t)nb * nK * nR),
           oWT = ar.add(sizeof(float) * (size_t)nb * nK * nT), oBL = ar.add(sizeof(float) * nb);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    float* A = (float*)ws_get(c, WS_A, sizeof(float) * (size_t)nb * nT * Kp, &st);
    if (!A) return st;
    float* D = (float*)ws_get(c, WS_D, sizeof(float) * (size_t)nR * nb * nT, &st);
    if (!D) return st;
    TG3_CUDA(cudaMemcpyAsync(b + orp, rotP, sizeof(float) * 2 * (size_t)nR * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + otp, traP, sizeof(float) * 2 * (size_t)nT * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, pR, sizeof(double) * nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, pT, sizeof(double) * nT, cudaMemcpyHostToDevice, s));
    {
        dim3 g1((Kp / 2 + 255) / 256, nR);
        k_pad_rows<<<g1, 256, 0, s>>>((const float2*)(b + orp), K, (float2*)P, Kp / 2);
        dim3 g2((Kq + 255) / 256, nR);
        k_abs2_rows<<<g2, 256, 0, s>>>((const float2*)(b + orp), K, nR, P2, Kq);
        TG3_LAUNCH_CHECK("bank preparation");
    }
    for (int l0 = 0; l0 < imgNum; l0 += IB) {
        const int n = std::min(IB, imgNum - l0);
        TG3_CUDA(cudaMemcpyAsync(b + od, datP + 2 * (size_t)l0 * K, sizeof(float) * 2 * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + oc, ctfP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + os, sigRcpP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        if (kIdx > 0) {
            TG3_CUDA(cudaMemcpyAsync(b + oWC, wC + (size_t)l0 * nK, sizeof(float) * (size_t)n * nK,
                                     cudaMemcpyHostToDevice, s));
            TG3_CUDA(cudaMemcpyAsync(b + oWR, wR + (size_t)l0 * nK * nR, sizeof(float) * (size_t)n * nK * nR,
                                     cudaMemcpyHostToDevice, s));
            TG3_CUDA(cudaMemcpyAsync(b + oWT, wT + (size_t)l0 * nK * nT, sizeof(float) * (size_t)n * nK * nT,
                                     cudaMemcpyHostToDevice, s));
            TG3_CUDA(cudaMemcpyAsync(b + oBL, baseL + l0, sizeof(float) * n, cudaMemcpyHostToDevice, s));
        }
        const float2* dd = (const float2*)(b + od);
        const float* cc = (const float*)(b + oc);
        const float* ss = (const float*)(b + os);
        TG3_CUDA(launch_shift_bank(dd, cc, ss, nullptr, (const float2*)(b + otp), n, nT, 1, nullptr,
                                   nullptr, K, A, Kp, 0, s));
        TG3_CUDA(launch_x0(dd, ss, n, K, (double*)(b + ox0), s));
        {
            dim3 g3((Kq + 255) / 256, n);
            k_sc2_rows<<<g3, 256, 0, s>>>(ss, cc, K, (float*)(b + osc), Kq);
            TG3_LAUNCH_CHECK("norm operand");
        }
        // cross term, written image-major: D[l][r][t] = -2 sum A''[l t] . P[r]
        TG3_CUDA(launch_gemm_nt_fp32(P, 0, Kp, A, 0, Kp, nR, n * nT, Kp, 1, D, 0, nT, nullptr, 0,
                                     -2.0f, s, nT, (long long)nR * nT));
        // norm term: N[r][l] = sum_p |P_rp|^2 sigRcp_lp ctf_lp^2
        TG3_CUDA(launch_gemm_nt_fp32(P2, 0, Kq, (const float*)(b + osc), 0, Kq, nR, n, Kq, 1,
                                     (float*)(b + onr), 0, n, nullptr, 0, 1.0f, s));
        TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, n, (const float*)(b + onr), n,
                                (const double*)(b + ox0), (const double*)(b + opr), 0,
                                (const double*)(b + opt), 0, nullptr, (double*)(b + owc),
                                (double*)(b + owr), (double*)(b + owt), (double*)(b + obs), nullptr, s));
        TG3_CUDA(launch_merge_class(n, nK, kIdx, nR, nT, (const double*)(b + owc),
                                    (const double*)(b + owr), (const double*)(b + owt),
                                    (const double*)(b + obs), (float*)(b + oWC), (float*)(b + oWR),
                                    (float*)(b + oWT), (float*)(b + oBL), s));
        TG3_CUDA(cudaMemcpyAsync(wC + (size_t)l0 * nK, b + oWC, sizeof(float) * (size_t)n * nK,
                                 cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(wR + (size_t)l0 * nK * nR, b + oWR, sizeof(float) * (size_t)n * nK * nR,
                                 cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(wT + (size_t)l0 * nK * nT, b + oWT, sizeof(float) * (size_t)n * nK * nT,
                                 cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(baseL + l0, b + oBL, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
        if ((st = sync_and_check(c))) return st;
    }
    return TG3_OK;
}

static int insert_ft(float* F3D, float* T3D, double* O3D, int* counter, const float* datP,
                     const float* ctfP, const float* ctfaData, const double* offS,
                     const float* w, const double* nR, const double* nT, const double* nD,
                     const int* nC, const int* iCol, const int* iRow, float pixelSize,
                     int cSearch, int opf, int npxl, int mReco, int idim, int dimSize,
                     int imgNum, int kernel)
{
    if (!F3D || !T3D || !O3D || !counter || !datP || (!ctfP && !cSearch) || !offS || !w || !nR ||
        !nT || !iCol || !iRow)
        return fail(TG3_ERR_ARG, "null pointer");
    if (cSearch && (!ctfaData || !nD || !(pixelSize > 0)))
        return fail(TG3_ERR_ARG, "defocus search insertion needs ctfaData, nD and pixelSize");
    if (opf < 1 || npxl <= 0 || mReco <= 0 || idim <= 0 || imgNum <= 0 || dimSize != opf * idim)
        return fail(TG3_ERR_ARG, "bad InsertFT sizes (dimSize must equal opf * idim)");
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    // the reference hands the reconstructor's padded pixel indices (i * opf)
    std::vector<int> ic(npxl), ir(npxl);
    for (int p = 0; p < npxl; p++) {
        if (iCol[p] % opf || iRow[p] % opf)
            return fail(TG3_ERR_ARG, "InsertFT pixel indices must be multiples of opf");
        ic[p] = iCol[p] / opf;
        ir[p] = iRow[p] / opf;
    }
    if ((st = tg3_ctx_set_pixels(c, ic.data(), ir.data(), npxl, idim))) return st;
    if ((st = tg3_ctx_insert_begin(c, dimSize, opf))) return st;
    cudaStream_t s = c->stream;
    const size_t nvox = (size_t)dimSize * dimSize * (dimSize / 2 + 1);
    const int K = npxl;
    Arena ar(c, WS_H2D);
    const int IB = 4096;
    const int nb = std::min(imgNum, IB);
    // the defocus search: one CTF row per draw, made on the device from the
    // image's attributes with the draw's defocus factor (kernel_CalculateCTF)
    const size_t ctfRowsB = cSearch ? (size_t)nb * mReco : (size_t)nb;
    size_t od = ar.add(sizeof(float) * 2 * (size_t)nb * K), oc = ar.add(sizeof(float) * ctfRowsB * K),
           oq = ar.add(sizeof(double) * 4 * (size_t)nb * mReco), ot = ar.add(sizeof(double) * 2 * (size_t)nb * mReco),
           oo = ar.add(sizeof(double) * 2 * (size_t)nb), ow = ar.add(sizeof(float) * (size_t)nb),
           oO = ar.add(sizeof(double) * 3), on = ar.add(sizeof(int)),
           oa = ar.add(cSearch ? sizeof(float) * 7 * (size_t)nb : 0),
           oda = ar.add(cSearch ? sizeof(float) * 7 * (size_t)nb * mReco : 0),
           ond = ar.add(cSearch ? sizeof(double) * (size_t)nb * mReco : 0),
           onc = ar.add(nC ? sizeof(int) * (size_t)nb : 0);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    TG3_CUDA(cudaMemcpyAsync(b + oO, O3D, sizeof(double) * 3, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + on, counter, sizeof(int), cudaMemcpyHostToDevice, s));
    for (int l0 = 0; l0 < imgNum; l0 += IB) {
        const int n = std::min(IB, imgNum - l0);
        TG3_CUDA(cudaMemcpyAsync(b + od, datP + 2 * (size_t)l0 * K, sizeof(float) * 2 * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        if (cSearch) {
            TG3_CUDA(cudaMemcpyAsync(b + oa, ctfaData + 7 * (size_t)l0, sizeof(float) * 7 * (size_t)n,
                                     cudaMemcpyHostToDevice, s));
            TG3_CUDA(cudaMemcpyAsync(b + ond, nD + (size_t)l0 * mReco,
                                     sizeof(double) * (size_t)n * mReco, cudaMemcpyHostToDevice, s));
            TG3_CUDA(launch_draw_attr((const float*)(b + oa), (const double*)(b + ond), n * mReco,
                                      mReco, (float*)(b + oda), s));
            TG3_CUDA(launch_ctf((const float*)(b + oda), n * mReco, pixelSize, idim, c->px.iCol,
                                c->px.iRow, K, (float*)(b + oc), s));
        } else {
            TG3_CUDA(cudaMemcpyAsync(b + oc, ctfP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                     cudaMemcpyHostToDevice, s));
        }
        TG3_CUDA(cudaMemcpyAsync(b + oq, nR + 4 * (size_t)l0 * mReco, sizeof(double) * 4 * (size_t)n * mReco,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + ot, nT + 2 * (size_t)l0 * mReco, sizeof(double) * 2 * (size_t)n * mReco,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + oo, offS + 2 * (size_t)l0, sizeof(double) * 2 * (size_t)n,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + ow, w + l0, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, s));
        if (nC)
            TG3_CUDA(cudaMemcpyAsync(b + onc, nC + l0, sizeof(int) * (size_t)n,
                                     cudaMemcpyHostToDevice, s));
        if ((st = insert_draws(c, n * mReco, mReco, (const float*)(b + od), (const float*)(b + oc),
                               (const double*)(b + oq), (const double*)(b + ot),
                               (const double*)(b + oo), (const float*)(b + ow), kernel,
                               (double*)(b + oO), (int*)(b + on), cSearch ? n * mReco : 0,
                               nC ? (const int*)(b + onc) : nullptr)))
            return st;
        // the staging buffer is reused by the next pass
        TG3_CUDA(cudaStreamSynchronize(s));
    }
    // add the accumulator to the caller's volumes
    float* dF = (float*)ws_get(c, WS_D2H, sizeof(float) * 3 * nvox, &st);
    if (!dF) return st;
    float* dT = dF + 2 * nvox;
    TG3_CUDA(cudaMemcpyAsync(dF, F3D, sizeof(float) * 2 * nvox, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(dT, T3D, sizeof(float) * nvox, cudaMemcpyHostToDevice, s));
    if ((st = tg3_ctx_insert_read_d(c, dF, dT, 1))) return st;
    TG3_CUDA(cudaMemcpyAsync(F3D, dF, sizeof(float) * 2 * nvox, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(T3D, dT, sizeof(float) * nvox, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(O3D, b + oO, sizeof(double) * 3, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(counter, b + on, sizeof(int), cudaMemcpyDeviceToHost, s));
    return sync_and_check(c);
}

extern "C" int tg3_InsertFT(float* F3D, float* T3D, double* O3D, int* counter, const float* datP,
                            const float* ctfP, const float* sigRcpP, const float* ctfaData,
                            const double* offS, const float* w, const double* nR,
                            const double* nT, const double* nD, const int* iCol, const int* iRow,
                            float pixelSize, int cSearch, int opf, int npxl, int mReco, int idim,
                            int dimSize, int imgNum, int kernel)
{
    (void)sigRcpP;
    return insert_ft(F3D, T3D, O3D, counter, datP, ctfP, ctfaData, offS, w, nR, nT, nD, nullptr,
                     iCol, iRow, pixelSize, cSearch, opf, npxl, mReco, idim, dimSize, imgNum,
                     kernel);
}

extern "C" int tg3_InsertFT_classes(float* F3D, float* T3D, double* O3D, int* counter,
                                    const float* datP, const float* ctfP, const float* sigRcpP,
                                    const float* ctfaData, const double* offS, const float* w,
                                    const double* nR, const double* nT, const double* nD,
                                    const int* nC, const int* iCol, const int* iRow,
                                    float pixelSize, int cSearch, int opf, int npxl, int mReco,
                                    int idim, int dimSize, int imgNum, int kernel)
{
    (void)sigRcpP;
    if (!nC) return fail(TG3_ERR_ARG, "null nC");
    for (int l = 0; l < imgNum; l++)
        if (nC[l] < 0 || nC[l] > mReco)
            return fail(TG3_ERR_ARG, "nC[l] must lie in [0, mReco]");
    return insert_ft(F3D, T3D, O3D, counter, datP, ctfP, ctfaData, offS, w, nR, nT, nD, nC,
                     iCol, iRow, pixelSize, cSearch, opf, npxl, mReco, idim, dimSize, imgNum,
                     kernel);
}

// ====================================================== volume handle + local
extern "C" int tg3_volume_create(tg3_volume** out, const float* volume, int vdim, int pf)
{
    if (!out) return fail(TG3_ERR_ARG, "null output");
    *out = nullptr;
    int dev = 0;
    TG3_CUDA(cudaGetDevice(&dev));
    tg3_volume* h = new tg3_volume();
    int st = tg3_ctx_create(&h->ctx, dev);
    if (st == TG3_OK) st = tg3_ctx_set_volume(h->ctx, 0, volume, vdim, pf, 0);
    if (st != TG3_OK) {
        tg3_ctx_destroy(h->ctx);
        delete h;
        return st;
    }
    *out = h;
    return TG3_OK;
}

extern "C" int tg3_volume_destroy(tg3_volume* h)
{
    if (!h) return TG3_OK;
    tg3_ctx_destroy(h->ctx);
    delete h;
    return TG3_OK;
}

extern "C" int tg3_ExpectLocal3D(tg3_volume* h, const float* dat, const float* ctf,
                                 const float* sigRcp, const int* iCol, const int* iRow, int npxl,
                                 int idim, const double* rot, int nR, const double* trans, int nT,
                                 const double* oldR, const double* oldT, double oldC, float* wC,
                                 float* wR, float* wT, float* dvp, float* baseL)
{
    if (!h || !h->ctx) return fail(TG3_ERR_ARG, "null volume handle");
    if (!dat || !ctf || !sigRcp || !iCol || !iRow || !rot || !trans || !oldR || !oldT || !wC ||
        !wR || !wT || !baseL || npxl <= 0 || nR <= 0 || nT <= 0)
        return fail(TG3_ERR_ARG, "bad ExpectLocal3D args");
    tg3_ctx* c = h->ctx;
    int st = check_ctx(c);
    if (st) return st;
    if (c->px.K != npxl || c->px.idim != idim) {
        if ((st = tg3_ctx_set_pixels(c, iCol, iRow, npxl, idim))) return st;
    }
    cudaStream_t s = c->stream;
    const int K = npxl;
    Arena ar(c, WS_H2D);
    size_t od = ar.add(8 * (size_t)K), oc = ar.add(4 * (size_t)K), os = ar.add(4 * (size_t)K),
           oq = ar.add(32 * (size_t)nR), ot = ar.add(16 * (size_t)nT), opr = ar.add(8 * (size_t)nR),
           opt = ar.add(8 * (size_t)nT), opc = ar.add(8), owc = ar.add(8), owr = ar.add(8 * (size_t)nR),
           owt = ar.add(8 * (size_t)nT), obl = ar.add(8), odv = ar.add(4 * (size_t)nR * nT);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    TG3_CUDA(cudaMemcpyAsync(b + od, dat, 8 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oc, ctf, 4 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + os, sigRcp, 4 * (size_t)K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oq, rot, 32 * (size_t)nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ot, trans, 16 * (size_t)nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, oldR, 8 * (size_t)nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, oldT, 8 * (size_t)nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opc, &oldC, 8, cudaMemcpyHostToDevice, s));
    st = local_phase(c, nullptr, 1, nR, nT, (float*)(b + od), (float*)(b + oc), (float*)(b + os),
                     (double*)(b + oq), (double*)(b + ot), (double*)(b + opr), (double*)(b + opt),
                     (double*)(b + opc), nullptr, (double*)(b + owc), (double*)(b + owr),
                     (double*)(b + owt), (double*)(b + obl), dvp ? (float*)(b + odv) : nullptr,
                     TG3_SCORE_FP32);
    if (st) return st;
    std::vector<double> hwr(nR), hwt(nT);
    double hwc = 0, hbl = 0;
    TG3_CUDA(cudaMemcpyAsync(hwr.data(), b + owr, 8 * (size_t)nR, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(hwt.data(), b + owt, 8 * (size_t)nT, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hwc, b + owc, 8, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hbl, b + obl, 8, cudaMemcpyDeviceToHost, s));
    if (dvp) TG3_CUDA(cudaMemcpyAsync(dvp, b + odv, 4 * (size_t)nR * nT, cudaMemcpyDeviceToHost, s));
    if ((st = sync_and_check(c))) return st;
    for (int r = 0; r < nR; r++) wR[r] = (float)hwr[r];
    for (int t = 0; t < nT; t++) wT[t] = (float)hwt[t];
    *wC = (float)hwc;
    *baseL = (float)hbl;
    return TG3_OK;
}

// The defocus-search form of tg3_ExpectLocal3D: the particle's CTF for each
// defocus factor dpara[d] from its per-pixel defocus defO and frequency freQ
// (kernel_CalCTFL), then the local phase over rotation x translation x
// defocus; wD[d] as wR / wT.
extern "C" int tg3_ExpectLocal3D_ctf(tg3_volume* h, const float* dat, const float* defO,
                                     const float* freQ, float k1, float k2, float phaseShift,
                                     float conT, const float* sigRcp, const int* iCol,
                                     const int* iRow, int npxl, int idim, const double* rot,
                                     int nR, const double* trans, int nT, const double* dpara,
                                     int nD, const double* oldR, const double* oldT,
                                     const double* oldD, double oldC, float* wC, float* wR,
                                     float* wT, float* wD, float* dvp, float* baseL)
{
    if (!h || !h->ctx) return fail(TG3_ERR_ARG, "null volume handle");
    if (!dat || !defO || !freQ || !sigRcp || !iCol || !iRow || !rot || !trans || !dpara ||
        !oldR || !oldT || !oldD || !wC || !wR || !wT || !wD || !baseL || npxl <= 0 || nR <= 0 ||
        nT <= 0 || nD < 1 || nD > 16)
        return fail(TG3_ERR_ARG, "bad ExpectLocal3D_ctf args");
    tg3_ctx* c = h->ctx;
    int st = check_ctx(c);
    if (st) return st;
    if (c->px.K != npxl || c->px.idim != idim) {
        if ((st = tg3_ctx_set_pixels(c, iCol, iRow, npxl, idim))) return st;
    }
    cudaStream_t s = c->stream;
    const size_t K = npxl, R_ = nR, T_ = nT, D_ = nD;
    Arena ar(c, WS_H2D);
    size_t od = ar.add(8 * K), odo = ar.add(4 * K), ofq = ar.add(4 * K), os = ar.add(4 * K),
           octf = ar.add(4 * K * D_), oq = ar.add(32 * R_), ot = ar.add(16 * T_),
           odp = ar.add(8 * D_), opr = ar.add(8 * R_), opt = ar.add(8 * T_), opd = ar.add(8 * D_),
           opc = ar.add(8), owc = ar.add(8), owr = ar.add(8 * R_), owt = ar.add(8 * T_),
           owd = ar.add(8 * D_), obl = ar.add(8), odv = ar.add(dvp ? 4 * D_ * R_ * T_ : 0);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    TG3_CUDA(cudaMemcpyAsync(b + od, dat, 8 * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + odo, defO, 4 * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ofq, freQ, 4 * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + os, sigRcp, 4 * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oq, rot, 32 * R_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ot, trans, 16 * T_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + odp, dpara, 8 * D_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, oldR, 8 * R_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, oldT, 8 * T_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opd, oldD, 8 * D_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opc, &oldC, 8, cudaMemcpyHostToDevice, s));
    TG3_CUDA(launch_ctf_defocus((float*)(b + odo), (float*)(b + ofq), (double*)(b + odp), nD,
                                npxl, k1, k2, phaseShift, conT, (float*)(b + octf), s));
    st = local_phase_ctf(c, 1, nR, nT, nD, (float*)(b + od), (float*)(b + octf), (float*)(b + os),
                         (double*)(b + oq), (double*)(b + ot), (double*)(b + opr),
                         (double*)(b + opt), (double*)(b + opd), (double*)(b + opc), nullptr,
                         (double*)(b + owc), (double*)(b + owr), (double*)(b + owt),
                         (double*)(b + owd), (double*)(b + obl), dvp ? (float*)(b + odv) : nullptr,
                         TG3_SCORE_FP32);
    if (st) return st;
    std::vector<double> hwr(R_), hwt(T_), hwd(D_);
    double hwc = 0, hbl = 0;
    TG3_CUDA(cudaMemcpyAsync(hwr.data(), b + owr, 8 * R_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(hwt.data(), b + owt, 8 * T_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(hwd.data(), b + owd, 8 * D_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hwc, b + owc, 8, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(&hbl, b + obl, 8, cudaMemcpyDeviceToHost, s));
    if (dvp) TG3_CUDA(cudaMemcpyAsync(dvp, b + odv, 4 * D_ * R_ * T_, cudaMemcpyDeviceToHost, s));
    if ((st = sync_and_check(c))) return st;
    for (int r = 0; r < nR; r++) wR[r] = (float)hwr[r];
    for (int t = 0; t < nT; t++) wT[t] = (float)hwt[t];
    for (int d = 0; d < nD; d++) wD[d] = (float)hwd[d];
    *wC = (float)hwc;
    *baseL = (float)hbl;
    return TG3_OK;
}

static int global_scan(tg3_ctx* c, const Volume* v, const float2* img2, int vdim, int pf,
                       int nImg, int nR, int nT, const float* dat, const float* ctf,
                       const float* sigRcp, const double* rotMat, const double* trans,
                       const double* pR, const double* pT, double* wC, double* wR, double* wT,
                       double* baseL, float* dvp, int precision, int nK = 1,
                       size_t imgStride = 0, Bank* pbank = nullptr);
static int merge_classes(tg3_ctx* c, int n, int nK, int nR, int nT, const double* wCd,
                         const double* wRd, const double* wTd, const double* bd, float* wC,
                         float* wR, float* wT, float* baseL);

// 2-D classification's global search (ExpectGlobal2D,
// gpu/interface/Interface.h:176-197; expectGlobal2D, gpu/src/cuthunder.cu:
// 889-): every image against nK class images at nR in-plane rotations x nT
// translations, the classes merged to each image's best hypothesis as the
// reference's running baseline does.  FP32, the reference's plain path.
extern "C" int tg3_ExpectGlobal2D(const float* vol, const float* datP, const float* ctfP,
                                  const float* sigRcpP, const double* trans, float* wC, float* wR,
                                  float* wT, const double* pR, const double* pT, const double* rot,
                                  const int* iCol, const int* iRow, int nK, int nR, int nT,
                                  int pf, int interp, int idim, int vdim, int npxl, int imgNum)
{
    if (!vol || !datP || !ctfP || !sigRcpP || !trans || !wC || !wR || !wT || !pR || !pT || !rot ||
        !iCol || !iRow)
        return fail(TG3_ERR_ARG, "null pointer");
    if (nK <= 0 || nK > 6144 || nR <= 0 || nT <= 0 || npxl <= 0 || imgNum <= 0 || pf < 1 ||
        vdim < 4 || (vdim & 1) || nT > 2048)
        return fail(TG3_ERR_ARG, "bad ExpectGlobal2D sizes");
    if (interp != 1) return fail(TG3_ERR_UNSUPPORTED, "only linear interpolation");
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    if ((st = tg3_ctx_set_pixels(c, iCol, iRow, npxl, idim))) return st;
    cudaStream_t s = c->stream;
    const int K = npxl;
    const size_t img = (size_t)vdim * (vdim / 2 + 1);
    const int IB = 1024;
    const int nb = std::min(imgNum, IB);
    Arena ar(c, WS_H2D);
    size_t oim = ar.add(sizeof(float) * 2 * img * nK), orot = ar.add(sizeof(double) * 2 * nR),
           otr = ar.add(sizeof(double) * 2 * nT), opr = ar.add(sizeof(double) * nR),
           opt = ar.add(sizeof(double) * nT), od = ar.add(sizeof(float) * 2 * (size_t)nb * K),
           oc = ar.add(sizeof(float) * (size_t)nb * K), os = ar.add(sizeof(float) * (size_t)nb * K),
           owc = ar.add(sizeof(double) * (size_t)nb * nK),
           owr = ar.add(sizeof(double) * (size_t)nb * nK * nR),
           owt = ar.add(sizeof(double) * (size_t)nb * nK * nT),
           obs = ar.add(sizeof(double) * (size_t)nb * nK),
           oWC = ar.add(sizeof(float) * (size_t)nb * nK),
           oWR = ar.add(sizeof(float) * (size_t)nb * nK * nR),
           oWT = ar.add(sizeof(float) * (size_t)nb * nK * nT), oBL = ar.add(sizeof(float) * nb);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    TG3_CUDA(cudaMemcpyAsync(b + oim, vol, sizeof(float) * 2 * img * nK, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + orot, rot, sizeof(double) * 2 * nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + otr, trans, sizeof(double) * 2 * nT, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, pR, sizeof(double) * nR, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, pT, sizeof(double) * nT, cudaMemcpyHostToDevice, s));
    for (int l0 = 0; l0 < imgNum; l0 += IB) {
        const int n = std::min(IB, imgNum - l0);
        TG3_CUDA(cudaMemcpyAsync(b + od, datP + 2 * (size_t)l0 * K, sizeof(float) * 2 * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + oc, ctfP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + os, sigRcpP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        // every class in one scan: one shifted-data bank, one cross-term GEMM
        st = global_scan(c, nullptr, (const float2*)(b + oim), vdim, pf, n, nR, nT,
                         (const float*)(b + od), (const float*)(b + oc), (const float*)(b + os),
                         (const double*)(b + orot), (const double*)(b + otr),
                         (const double*)(b + opr), (const double*)(b + opt), (double*)(b + owc),
                         (double*)(b + owr), (double*)(b + owt), (double*)(b + obs), nullptr,
                         TG3_SCORE_FP32, nK, img);
        if (st) return st;
        if ((st = merge_classes(c, n, nK, nR, nT, (const double*)(b + owc),
                                (const double*)(b + owr), (const double*)(b + owt),
                                (const double*)(b + obs), (float*)(b + oWC), (float*)(b + oWR),
                                (float*)(b + oWT), (float*)(b + oBL))))
            return st;
        TG3_CUDA(cudaMemcpyAsync(wC + (size_t)l0 * nK, b + oWC, sizeof(float) * (size_t)n * nK,
                                 cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(wR + (size_t)l0 * nK * nR, b + oWR,
                                 sizeof(float) * (size_t)n * nK * nR, cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(wT + (size_t)l0 * nK * nT, b + oWT,
                                 sizeof(float) * (size_t)n * nK * nT, cudaMemcpyDeviceToHost, s));
        // the staging buffer is reused by the next pass
        if ((st = sync_and_check(c))) return st;
    }
    return TG3_OK;
}

// 2-D classification's insertion, InsertI2D (gpu/interface/Interface.h:
// 239-266, without its communicators): every draw into the accumulator of
// its class; F2D / T2D [nk][vdim][vdim/2 + 1] accumulated into, O2D [nk][2]
// and counter [nk] added to.  iCol / iRow are the reconstructor's padded
// indices (i opf).  With cSearch each draw's CTF is made from its image's
// CTFAttr and the draw's defocus factor nD, as in tg3_InsertFT.
extern "C" int tg3_InsertI2D(float* F2D, float* T2D, double* O2D, int* counter,
                             const float* datP, const float* ctfP, const float* sigRcpP,
                             const float* w, const double* offS, const int* nC, const double* nR,
                             const double* nT, const double* nD, const float* ctfaData,
                             const int* iCol, const int* iRow, float pixelSize, int cSearch,
                             int nk, int opf, int npxl, int mReco, int idim, int vdim,
                             int imgNum)
{
    (void)sigRcpP;
    if (!F2D || !T2D || !O2D || !counter || !datP || (!ctfP && !cSearch) || !w || !offS ||
        !nC || !nR || !nT || !iCol || !iRow)
        return fail(TG3_ERR_ARG, "null pointer");
    if (cSearch && (!ctfaData || !nD || !(pixelSize > 0)))
        return fail(TG3_ERR_ARG, "defocus search insertion needs ctfaData, nD and pixelSize");
    if (nk <= 0 || opf < 1 || npxl <= 0 || mReco <= 0 || idim <= 0 || imgNum <= 0 ||
        vdim != opf * idim)
        return fail(TG3_ERR_ARG, "bad InsertI2D sizes (vdim must equal opf * idim)");
    for (int d = 0; d < imgNum * mReco; d++)
        if (nC[d] < 0 || nC[d] >= nk) return fail(TG3_ERR_ARG, "class index out of range");
    int st = TG3_OK;
    tg3_ctx* c = default_ctx(&st);
    if (!c) return st;
    std::vector<int> ic(npxl), ir(npxl);
    for (int p = 0; p < npxl; p++) {
        if (iCol[p] % opf || iRow[p] % opf)
            return fail(TG3_ERR_ARG, "InsertI2D pixel indices must be multiples of opf");
        ic[p] = iCol[p] / opf;
        ir[p] = iRow[p] / opf;
    }
    if ((st = tg3_ctx_set_pixels(c, ic.data(), ir.data(), npxl, idim))) return st;
    if ((st = check_geometry(c, vdim, opf, 1.0))) return st;
    cudaStream_t s = c->stream;
    const size_t nvox = (size_t)vdim * (vdim / 2 + 1);
    const int K = npxl;
    const int IB = 4096;
    const int nb = std::min(imgNum, IB);
    const size_t ctfRowsB = cSearch ? (size_t)nb * mReco : (size_t)nb;
    Arena ar(c, WS_H2D);
    size_t oacc = ar.add(sizeof(float4) * nvox * nk), od = ar.add(sizeof(float) * 2 * (size_t)nb * K),
           oc = ar.add(sizeof(float) * ctfRowsB * K), ow = ar.add(sizeof(float) * nb),
           oo = ar.add(sizeof(double) * 2 * nb), onc = ar.add(sizeof(int) * (size_t)nb * mReco),
           onr = ar.add(sizeof(double) * 2 * (size_t)nb * mReco),
           ont = ar.add(sizeof(double) * 2 * (size_t)nb * mReco), oO = ar.add(sizeof(double) * 2 * nk),
           ocn = ar.add(sizeof(int) * nk), oa = ar.add(cSearch ? sizeof(float) * 7 * (size_t)nb : 0),
           oda = ar.add(cSearch ? sizeof(float) * 7 * (size_t)nb * mReco : 0),
           ond = ar.add(cSearch ? sizeof(double) * (size_t)nb * mReco : 0),
           oF = ar.add(sizeof(float) * 2 * nvox), oT = ar.add(sizeof(float) * nvox);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    float4* acc = (float4*)(b + oacc);
    TG3_CUDA(cudaMemsetAsync(acc, 0, sizeof(float4) * nvox * nk, s));
    TG3_CUDA(cudaMemcpyAsync(b + oO, O2D, sizeof(double) * 2 * nk, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ocn, counter, sizeof(int) * nk, cudaMemcpyHostToDevice, s));
    for (int l0 = 0; l0 < imgNum; l0 += IB) {
        const int n = std::min(IB, imgNum - l0);
        const size_t nd = (size_t)n * mReco, d0 = (size_t)l0 * mReco;
        TG3_CUDA(cudaMemcpyAsync(b + od, datP + 2 * (size_t)l0 * K, sizeof(float) * 2 * (size_t)n * K,
                                 cudaMemcpyHostToDevice, s));
        if (cSearch) {
            TG3_CUDA(cudaMemcpyAsync(b + oa, ctfaData + 7 * (size_t)l0, sizeof(float) * 7 * (size_t)n,
                                     cudaMemcpyHostToDevice, s));
            TG3_CUDA(cudaMemcpyAsync(b + ond, nD + d0, sizeof(double) * nd, cudaMemcpyHostToDevice, s));
            TG3_CUDA(launch_draw_attr((const float*)(b + oa), (const double*)(b + ond), (int)nd,
                                      mReco, (float*)(b + oda), s));
            TG3_CUDA(launch_ctf((const float*)(b + oda), (int)nd, pixelSize, idim, c->px.iCol,
                                c->px.iRow, K, (float*)(b + oc), s));
        } else {
            TG3_CUDA(cudaMemcpyAsync(b + oc, ctfP + (size_t)l0 * K, sizeof(float) * (size_t)n * K,
                                     cudaMemcpyHostToDevice, s));
        }
        TG3_CUDA(cudaMemcpyAsync(b + ow, w + l0, sizeof(float) * n, cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + oo, offS + 2 * (size_t)l0, sizeof(double) * 2 * n,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + onc, nC + d0, sizeof(int) * nd, cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + onr, nR + 2 * d0, sizeof(double) * 2 * nd, cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + ont, nT + 2 * d0, sizeof(double) * 2 * nd, cudaMemcpyHostToDevice, s));
        TG3_CUDA(launch_insert2d(acc, vdim, (const float2*)(b + od), (const float*)(b + oc),
                                 cSearch ? 1 : 0, (const float*)(b + ow), (const double*)(b + oo),
                                 (const int*)(b + onc), (const double*)(b + onr),
                                 (const double*)(b + ont), c->px.iCol, c->px.iRow, K, opf, idim,
                                 (int)nd, mReco, (double*)(b + oO), (int*)(b + ocn), s));
        // the staging buffers are reused by the next pass
        TG3_CUDA(cudaStreamSynchronize(s));
    }
    // add every class's accumulator to the caller's volumes
    for (int k = 0; k < nk; k++) {
        TG3_CUDA(cudaMemcpyAsync(b + oF, F2D + 2 * nvox * k, sizeof(float) * 2 * nvox,
                                 cudaMemcpyHostToDevice, s));
        TG3_CUDA(cudaMemcpyAsync(b + oT, T2D + nvox * k, sizeof(float) * nvox, cudaMemcpyHostToDevice,
                                 s));
        TG3_CUDA(launch_acc_read(acc + nvox * k, nvox, (float2*)(b + oF), (float*)(b + oT), 1, s));
        TG3_CUDA(cudaMemcpyAsync(F2D + 2 * nvox * k, b + oF, sizeof(float) * 2 * nvox,
                                 cudaMemcpyDeviceToHost, s));
        TG3_CUDA(cudaMemcpyAsync(T2D + nvox * k, b + oT, sizeof(float) * nvox, cudaMemcpyDeviceToHost,
                                 s));
        TG3_CUDA(cudaStreamSynchronize(s));
    }
    TG3_CUDA(cudaMemcpyAsync(O2D, b + oO, sizeof(double) * 2 * nk, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(counter, b + ocn, sizeof(int) * nk, cudaMemcpyDeviceToHost, s));
    return sync_and_check(c);
}

// ====================================================== host batched phase
extern "C" int tg3_local_phase(tg3_ctx* c, int nP, int nR, int nT, const float* dat,
                               const float* ctf, const float* sigRcp, const double* quat,
                               const double* trans, const double* pwR, const double* pwT,
                               const double* pwC, const int* cls, double* wC, double* wR,
                               double* wT, double* baseL, float* dvp, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (nP <= 0 || nR <= 0 || nT <= 0 || nT > 2048) return fail(TG3_ERR_ARG, "bad batch shape (nT <= 2048)");
    if (!dat || !ctf || !sigRcp || !quat || !trans || !pwR || !pwT || !wC || !wR || !wT || !baseL)
        return fail(TG3_ERR_ARG, "null host pointer");
    const size_t K = c->px.K;
    if (K == 0) return fail(TG3_ERR_STATE, "pixel list not set");
    Arena ar(c, WS_H2D);
    const size_t P_ = nP, R_ = nR, T_ = nT;
    size_t od = ar.add(8 * P_ * K), oc = ar.add(4 * P_ * K), os = ar.add(4 * P_ * K),
           oq = ar.add(32 * P_ * R_), ot = ar.add(16 * P_ * T_), opr = ar.add(8 * P_ * R_),
           opt = ar.add(8 * P_ * T_), opc = ar.add(8 * P_), ocl = ar.add(4 * P_),
           owc = ar.add(8 * P_), owr = ar.add(8 * P_ * R_), owt = ar.add(8 * P_ * T_),
           obl = ar.add(8 * P_), odv = ar.add(dvp ? 4 * P_ * R_ * T_ : 0);
    char* b = (char*)ws_get(c, WS_H2D, ar.used, &st);
    if (!b) return st;
    cudaStream_t s = c->stream;
    TG3_CUDA(cudaMemcpyAsync(b + od, dat, 8 * P_ * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oc, ctf, 4 * P_ * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + os, sigRcp, 4 * P_ * K, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + oq, quat, 32 * P_ * R_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + ot, trans, 16 * P_ * T_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opr, pwR, 8 * P_ * R_, cudaMemcpyHostToDevice, s));
    TG3_CUDA(cudaMemcpyAsync(b + opt, pwT, 8 * P_ * T_, cudaMemcpyHostToDevice, s));
    if (pwC) TG3_CUDA(cudaMemcpyAsync(b + opc, pwC, 8 * P_, cudaMemcpyHostToDevice, s));
    if (cls) TG3_CUDA(cudaMemcpyAsync(b + ocl, cls, 4 * P_, cudaMemcpyHostToDevice, s));
    st = local_phase(c, nullptr, nP, nR, nT, (float*)(b + od), (float*)(b + oc), (float*)(b + os),
                     (double*)(b + oq), (double*)(b + ot), (double*)(b + opr), (double*)(b + opt),
                     pwC ? (double*)(b + opc) : nullptr, cls ? (int*)(b + ocl) : nullptr,
                     (double*)(b + owc), (double*)(b + owr), (double*)(b + owt),
                     (double*)(b + obl), dvp ? (float*)(b + odv) : nullptr, precision);
    if (st) return st;
    TG3_CUDA(cudaMemcpyAsync(wC, b + owc, 8 * P_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(wR, b + owr, 8 * P_ * R_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(wT, b + owt, 8 * P_ * T_, cudaMemcpyDeviceToHost, s));
    TG3_CUDA(cudaMemcpyAsync(baseL, b + obl, 8 * P_, cudaMemcpyDeviceToHost, s));
    if (dvp) TG3_CUDA(cudaMemcpyAsync(dvp, b + odv, 4 * P_ * R_ * T_, cudaMemcpyDeviceToHost, s));
    return sync_and_check(c);
}

// ============================================================ stage timing
extern "C" int tg3_ctx_set_option(tg3_ctx* c, int option, int value)
{
    int st = check_ctx(c);
    if (st) return st;
    if (option == TG3_OPT_FUSED) c->fused = value != 0;
    else if (option == TG3_OPT_INSERT_GATHER) c->insertGather = value != 0;
    else if (option == TG3_OPT_BANK_GATHER) {
        if (value < 0 || value > 2) return fail(TG3_ERR_ARG, "TG3_OPT_BANK_GATHER takes 0, 1 or 2");
        c->bankGather = value;
    }
    else if (option == TG3_OPT_BANK_ORDER) c->bankOrder = value != 0;
    else if (option == TG3_OPT_SCAN_TILE_N) {
        if (value != 0 && (value < 16 || value > 256 || value % 16))
            return fail(TG3_ERR_ARG, "TG3_OPT_SCAN_TILE_N takes 0 or a multiple of 16 up to 256");
        c->scanTileN = value;
    }
    else if (option == TG3_OPT_SCAN_PAIR) c->scanPair = value != 0;
    else if (option == TG3_OPT_SCAN_BK) {
        if (value != 32 && value != 64) return fail(TG3_ERR_ARG, "TG3_OPT_SCAN_BK takes 32 or 64");
        c->scanBK = value;
    }
    else if (option == TG3_OPT_LOCAL_BK) {
        if (value != 32 && value != 64) return fail(TG3_ERR_ARG, "TG3_OPT_LOCAL_BK takes 32 or 64");
        c->localBK = value;
    }
    else if (option == TG3_OPT_BANK_SHAPE) {
        if (value < 0 || value > 3) return fail(TG3_ERR_ARG, "TG3_OPT_BANK_SHAPE takes 0 to 3");
        c->bankShape = value;
    }
    else if (option == TG3_OPT_PROJECT_GROUP) {
        if (value != 4 && value != 8 && value != 16)
            return fail(TG3_ERR_ARG, "TG3_OPT_PROJECT_GROUP takes 4, 8 or 16");
        c->projGroup = value;
    }
    else if (option == TG3_OPT_PROJECT_FORM) {
        if (value < 0 || value > 4) return fail(TG3_ERR_ARG, "TG3_OPT_PROJECT_FORM takes 0 to 4");
        c->projForm = value;
    }
    else return fail(TG3_ERR_ARG, "unknown option");
    return TG3_OK;
}

extern "C" int tg3_ctx_set_timing(tg3_ctx* c, int enable)
{
    int st = check_ctx(c);
    if (st) return st;
    c->timing = enable != 0;
    return TG3_OK;
}

extern "C" int tg3_ctx_stage_times(tg3_ctx* c, double* ms, int* launches, int reset)
{
    int st = check_ctx(c);
    if (st) return st;
    TG3_CUDA(cudaStreamSynchronize(c->stream));
    collect_times(c);
    for (int i = 0; i < TG3_STAGE_COUNT; i++) {
        if (ms) ms[i] = c->stageMs[i];
        if (launches) launches[i] = c->stageLaunches[i];
        if (reset) {
            c->stageMs[i] = 0;
            c->stageLaunches[i] = 0;
        }
    }
    return TG3_OK;
}

// ======================================================= global scan (device)
namespace tg3 {
// |P|^2 of padded projection rows (floats, or split bf16 planes with the lo
// plane loOff elements after the hi plane) into rows of ldq floats, or with
// outLo != 0 into split bf16 planes (hi = bf16(v), lo = bf16(v - hi), the lo
// plane outLo elements after the hi plane) for the tensor-core norm term.
__global__ void k_abs2_from(const float* __restrict__ P, long long loOff, int K, int Kp,
                            float* __restrict__ out, int ldq, long long outLo = 0)
{
    const int r = blockIdx.x;
    for (int p = threadIdx.x; p < ldq; p += blockDim.x) {
        float v = 0.f;
        if (p < K) {
            float re, im;
            if (loOff == 0) {
                const float2 a = reinterpret_cast<const float2*>(P + (size_t)r * Kp)[p];
                re = a.x;
                im = a.y;
            } else {
                const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(
                    reinterpret_cast<const __nv_bfloat16*>(P) + (size_t)r * Kp);
                const __nv_bfloat162* l = reinterpret_cast<const __nv_bfloat162*>(
                    reinterpret_cast<const __nv_bfloat16*>(P) + loOff + (size_t)r * Kp);
                const float2 hf = __bfloat1622float2(h[p]), lf = __bfloat1622float2(l[p]);
                re = hf.x + lf.x;
                im = hf.y + lf.y;
            }
            v = re * re + im * im;
        }
        if (outLo == 0) {
            out[(size_t)r * ldq + p] = v;
        } else {
            __nv_bfloat16* hi = reinterpret_cast<__nv_bfloat16*>(out);
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            hi[(size_t)r * ldq + p] = h;
            hi[outLo + (size_t)r * ldq + p] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

// sigRcp ctf^2 of every image's pixels as split bf16 planes [n][ldq] (hi,
// then lo outLo elements later), zero beyond K: the norm term's B operand.
__global__ void k_sc2_split(const float* __restrict__ sig, const float* __restrict__ ctf, int K,
                            __nv_bfloat16* __restrict__ hi, long long outLo, int ldq)
{
    const int r = blockIdx.y;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < ldq; p += gridDim.x * blockDim.x) {
        float v = 0.f;
        if (p < K) {
            const float c = ctf[(size_t)r * K + p];
            v = sig[(size_t)r * K + p] * c * c;
        }
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        hi[(size_t)r * ldq + p] = h;
        hi[outLo + (size_t)r * ldq + p] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
}
}  // namespace tg3

// The global scan of one class.  The projections come from the class's 3-D
// volume v at rotation matrices rot [nR][9], or (img2 != nullptr) from a 2-D
// class image img2 [vdim][vdim/2 + 1] at in-plane rotations rot [nR][2].
// The global scan of nImg images over nR rotations x nT translations.  With
// nK > 1 (2-D classes only: img2 holds nK class images imgStride complex
// values apart) every class's rotations are rows of one projection matrix,
// so the shifted-data bank is built once and one cross-term GEMM serves all
// classes; the weights are then per (image, class) block, each relative to
// its own best hypothesis: wC / baseL [nImg][nK], wR [nImg][nK][nR],
// wT [nImg][nK][nT], dvp [nImg][nK][nR][nT].
// nrmG [M][n] = sum_k abs2 [M][k] sc2 [n][k] over Kq columns: the FP32 GEMM,
// split along K into S chunks when its M x n tiles alone would not fill the
// GPU (the global search of a few fallback particles has n of about 70), the
// chunks' partial sums added in chunk order.
static int norm_gemm(tg3_ctx* c, const float* abs2, const float* sc2, int M, int n, int Kq,
                     float* nrmG, cudaStream_t s)
{
    const int tiles = ((M + 127) / 128) * ((n + 127) / 128);
    int S = 1;
    const int blocks64 = Kq / 64;
    if (tiles < 2 * 152 && Kq % 64 == 0) {
        const int want = std::min(16, (2 * 152 + tiles - 1) / tiles);
        for (int d = want; d >= 2; d--)
            if (blocks64 % d == 0) {
                S = d;
                break;
            }
    }
    if (S == 1) {
        TG3_CUDA(launch_gemm_nt_fp32(abs2, 0, Kq, sc2, 0, Kq, M, n, Kq, 1, nrmG, 0, n, nullptr, 0,
                                     1.0f, s));
        return TG3_OK;
    }
    int st = TG3_OK;
    const size_t cnt = (size_t)M * n;
    float* part = (float*)ws_get(c, WS_SPLITK, sizeof(float) * cnt * S, &st);
    if (!part) return st;
    const int kc = Kq / S;
    TG3_CUDA(launch_gemm_nt_fp32(abs2, kc, Kq, sc2, kc, Kq, M, n, kc, S, part, (long long)cnt, n,
                                 nullptr, 0, 1.0f, s));
    TG3_CUDA(launch_sum_parts(part, S, cnt, nrmG, s));
    return TG3_OK;
}

static int global_scan(tg3_ctx* c, const Volume* v, const float2* img2, int vdim, int pf,
                       int nImg, int nR, int nT, const float* dat, const float* ctf,
                       const float* sigRcp, const double* rotMat, const double* trans,
                       const double* pR, const double* pT, double* wC, double* wR, double* wT,
                       double* baseL, float* dvp, int precision, int nK, size_t imgStride,
                       Bank* pbank)
{
    int st = TG3_OK;
    if (pbank) {
        // the rotations are the bank's, already projected on the active pixels
        if (pbank->nB <= 0 || pbank->gen != c->px.gen || pbank->K != c->px.K)
            return fail(TG3_ERR_STATE, "no projection bank of the class on the active pixel set");
        nR = pbank->nB;
        nK = 1;
        img2 = nullptr;
        rotMat = pbank->quat;   // checked as non-null only
    }
    if (nImg <= 0 || nR <= 0 || nT <= 0 || nT > 2048) return fail(TG3_ERR_ARG, "bad scan shape");
    if (nK < 1 || (nK > 1 && !img2) || (long long)nK * nR > (1LL << 20))
        return fail(TG3_ERR_ARG, "bad class count");
    const int nRt = nK * nR;     // projected rows
    if (!dat || !ctf || !sigRcp || !rotMat || !trans || !pR || !pT || !wC || !wR || !wT || !baseL)
        return fail(TG3_ERR_ARG, "null device pointer");
    if (precision != TG3_SCORE_FP32 && precision != TG3_SCORE_BF16X3)
        return fail(TG3_ERR_ARG, "unknown precision");
    const bool split = precision == TG3_SCORE_BF16X3;
    if (split && !bf16x3_available()) return fail(TG3_ERR_UNSUPPORTED, "no TMA encoder");
    if ((st = check_geometry(c, vdim, pf))) return st;
    if ((st = check_weights_shape(nR, nT))) return st;
    const int K = c->px.K, Kp = c->px.Kp, Kq = (int)round_up(K, 64);
    // images per pass: keep the likelihood block within 4 GiB
    long long ib = (4LL << 30) / (4LL * nRt * nT);
    const int IB = (int)std::max(1LL, std::min(std::min((long long)nImg, ib), 65535LL));
    // workspace
    float* P = pbank ? (split ? reinterpret_cast<float*>(pbank->hi) : pbank->f32)
                    : (float*)ws_get(c, WS_P, 4 * (size_t)nRt * Kp, &st);
    if (!P) return st;
    float* A = (float*)ws_get(c, WS_A, 4 * (size_t)IB * nT * Kp, &st);
    if (!A) return st;
    float* D = (float*)ws_get(c, WS_D, 4 * (size_t)IB * nRt * nT, &st);
    if (!D) return st;
    float* nrmG = (float*)ws_get(c, WS_NRM, 4 * (size_t)nRt * IB, &st);
    if (!nrmG) return st;
    double* x0 = (double*)ws_get(c, WS_X0, 8 * (size_t)nImg, &st);
    if (!x0) return st;
    Arena ar(c, WS_MISC);
    const size_t oAbs = ar.add(pbank ? 0 : 4 * (size_t)nRt * Kq), oBank = ar.add(8 * (size_t)nT * K),
                 oSc = ar.add(4 * (size_t)IB * Kq),
                 oNc = ar.add(nK > 1 ? 4 * (size_t)nRt * IB : 0),
                 oX0 = ar.add(nK > 1 ? 8 * (size_t)IB * nK : 0);
    char* m = (char*)ws_get(c, WS_MISC, ar.used, &st);
    if (!m) return st;
    float* abs2 = pbank ? nullptr : (float*)(m + oAbs);
    float2* bank = (float2*)(m + oBank);
    float* sc2 = (float*)(m + oSc);
    float* nrmC = (float*)(m + oNc);
    double* x0r = (double*)(m + oX0);
    float* pscr = (img2 || pbank)
                      ? nullptr
                      : (float*)ws_get(c, WS_PROJ, sizeof(float) * project_scratch_floats(nR, Kp),
                                       &st);
    if (!img2 && !pbank && !pscr) return st;
    cudaStream_t s = c->stream;
    const long long splitP = split ? (long long)nRt * Kp : 0;
    {
        StageTimer tm(c, TG3_STAGE_PROJECT);
        if (pbank) {
            // the bank's planes are the projections (hi then lo: nB Kp apart)
        } else if (img2) {
            for (int k = 0; k < nK; k++) {
                // class k's rows start k nR rows in (bf16 rows in the split layout)
                const size_t off = (size_t)k * nR * Kp;
                float* Pk = split ? reinterpret_cast<float*>(reinterpret_cast<__nv_bfloat16*>(P) + off)
                                  : P + off;
                TG3_CUDA(launch_project2d(img2 + (size_t)k * imgStride, vdim, pf, rotMat, nR,
                                          c->px.iCol, c->px.iRow, K, Pk, Kp, splitP, s));
            }
        } else {
            TG3_CUDA(launch_project(nullptr, nullptr, v->blocks, v->vdim, v->pf, nullptr, rotMat,
                                    nR, nR, c->px.iCol, c->px.iRow, K, P, Kp, nullptr, nullptr,
                                    nullptr, pscr, c->d_flag, splitP, s, c->projForm, c->projGroup));
        }
        // |P|^2 rows: FP32 for the FP32 search, split bf16 planes (the same
        // bytes) for the split search's tensor-core norm term
        const long long outLo = split ? (long long)nRt * Kq : 0;
        if (pbank) {
            // the bank's, made once per bank and precision
            if (!pbank->abs2q)
                TG3_CUDA(cudaMalloc(&pbank->abs2q, sizeof(float) * (size_t)pbank->nB * Kq));
            if (pbank->abs2qSplit != (split ? 1 : 0)) {
                k_abs2_from<<<nRt, 256, 0, s>>>(P, splitP, K, Kp, pbank->abs2q, Kq, outLo);
                TG3_LAUNCH_CHECK("projection norms");
                pbank->abs2qSplit = split ? 1 : 0;
            }
            abs2 = pbank->abs2q;
        } else {
            k_abs2_from<<<nRt, 256, 0, s>>>(P, splitP, K, Kp, abs2, Kq, outLo);
            TG3_LAUNCH_CHECK("projection norms");
        }
    }
    TG3_CUDA(launch_translate(trans, nT, c->px.idim, c->px.iCol, c->px.iRow, K, bank, K, s));
    for (int l0 = 0; l0 < nImg; l0 += IB) {
        const int n = std::min(IB, nImg - l0);
        const float2* dd = reinterpret_cast<const float2*>(dat) + (size_t)l0 * K;
        const float* cc = ctf + (size_t)l0 * K;
        const float* ss = sigRcp + (size_t)l0 * K;
        const long long splitA = split ? (long long)n * nT * Kp : 0;
        {
            StageTimer tm(c, TG3_STAGE_SHIFT);
            TG3_CUDA(launch_shift_bank(dd, cc, ss, nullptr, bank, n, nT, 1, nullptr, nullptr, K, A,
                                       Kp, splitA, s));
            TG3_CUDA(launch_x0(dd, ss, n, K, x0 + l0, s));
            if (split)
                k_sc2_split<<<dim3((Kq + 255) / 256, n), 256, 0, s>>>(
                    ss, cc, K, reinterpret_cast<__nv_bfloat16*>(sc2), (long long)n * Kq, Kq);
            else
                k_sc2_rows<<<dim3((Kq + 255) / 256, n), 256, 0, s>>>(ss, cc, K, sc2, Kq);
            TG3_LAUNCH_CHECK("norm operand");
        }
        {
            // per-(rotation, image) norm: FP32 for the FP32 search; for the
            // split search the same three-product split-bf16 GEMM as the cross
            // term (|P|^2 and sigRcp ctf^2 are both split; FP32 accumulation)
            StageTimer tm(c, TG3_STAGE_NORM);
            if (split) {
                const int Nn = std::min(256, (n + 15) / 16 * 16);
                const int itemsN = (n + Nn - 1) / Nn;
                TG3_CUDA(launch_gemm_bf16x3(abs2, nRt, sc2, n, nRt, Nn, Kq, itemsN, 0, Nn, n, nrmG,
                                            Nn, n, nullptr, 0, 1.0f, c->d_flag, s, 0, 0, false,
                                            Kq % c->scanBK == 0 ? c->scanBK : 64));
            } else if ((st = norm_gemm(c, abs2, sc2, nRt, n, Kq, nrmG, s))) {
                return st;
            }
        }
        {
            StageTimer tm(c, TG3_STAGE_CROSS);
            // the cross term is written image-major: D[l][r][t]
            const int cols = n * nT;
            if (split) {
                const int Nt = std::min(c->scanTileN > 0 ? c->scanTileN : 256,
                                        (cols + 15) / 16 * 16);
                const int items = (cols + Nt - 1) / Nt;
                TG3_CUDA(launch_gemm_bf16x3(P, nRt, A, (long long)cols, nRt, Nt, Kp, items, 0, Nt,
                                            cols, D, 0, nT, nullptr, 0, -2.0f, c->d_flag, s, nT,
                                            (long long)nRt * nT, c->scanPair != 0,
                                            Kp % c->scanBK == 0 ? c->scanBK : 64));
            } else {
                TG3_CUDA(launch_gemm_nt_fp32(P, 0, Kp, A, 0, Kp, nRt, cols, Kp, 1, D, 0, nT,
                                             nullptr, 0, -2.0f, s, nT, (long long)nRt * nT));
            }
        }
        {
            StageTimer tm(c, TG3_STAGE_WEIGHTS);
            if (nK == 1) {
                // few images (the fallback particles of one class): each
                // image's rotations over several CTAs, so the GPU fills
                int nc = 1;
                if (n < 2 * 152 && nR >= 512)
                    nc = std::min(std::min(16, nR / 256), (2 * 152 + n - 1) / n);
                double* tmp = nullptr;
                if (nc > 1) {
                    tmp = (double*)ws_get(c, WS_WCHUNK,
                                          sizeof(double) * weights_chunk_doubles(n, nc, nT), &st);
                    if (!tmp) return st;
                }
                TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, n, nrmG, n, x0 + l0,
                                        pR, 0, pT, 0, nullptr, wC + l0, wR + (size_t)l0 * nR,
                                        wT + (size_t)l0 * nT, baseL + l0,
                                        dvp ? dvp + (size_t)l0 * nR * nT : nullptr, s, 512, nc,
                                        tmp));
            } else {
                // one block per (image, class): D[l][k nR + r][t] is block l nK + k
                const size_t b0 = (size_t)l0 * nK;
                TG3_CUDA(launch_nrm_classes(nrmG, nK, nR, n, nrmC, s));
                TG3_CUDA(launch_repeat_rows(x0 + l0, n, 1, nK, x0r, s));
                // many small blocks: 4 warps each when a class has few rotations
                TG3_CUDA(launch_weights(D, (long long)nR * nT, nT, nR, nT, 1, n * nK, nrmC, n * nK,
                                        x0r, pR, 0, pT, 0, nullptr, wC + b0, wR + b0 * nR,
                                        wT + b0 * nT, baseL + b0,
                                        dvp ? dvp + b0 * nR * nT : nullptr, s,
                                        nR < 128 ? 128 : (nR < 256 ? 256 : 512)));
            }
        }
    }
    return TG3_OK;
}

int tg3::global_scan_bank(tg3_ctx* c, int cls, int nImg, int nT, const float* dat,
                          const float* ctf, const float* sigRcp, const double* trans,
                          const double* pR, const double* pT, double* wC, double* wR,
                          double* wT, double* baseL, float* dvp, int precision)
{
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks)
        return fail(TG3_ERR_STATE, "volume of the class not set");
    const Volume& v = c->vol[cls];
    return global_scan(c, &v, nullptr, v.vdim, v.pf, nImg, 0, nT, dat, ctf, sigRcp, nullptr,
                       trans, pR, pT, wC, wR, wT, baseL, dvp, precision, 1, 0, &c->bank[cls]);
}

extern "C" int tg3_global_scan_d(tg3_ctx* c, int cls, int nImg, int nR, int nT, const float* dat,
                                 const float* ctf, const float* sigRcp, const double* rotMat,
                                 const double* trans, const double* pR, const double* pT,
                                 double* wC, double* wR, double* wT, double* baseL, float* dvp,
                                 int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (cls < 0 || cls >= kMaxClasses || !c->vol[cls].blocks)
        return fail(TG3_ERR_STATE, "volume of the class not set");
    const Volume& v = c->vol[cls];
    return global_scan(c, &v, nullptr, v.vdim, v.pf, nImg, nR, nT, dat, ctf, sigRcp, rotMat,
                       trans, pR, pT, wC, wR, wT, baseL, dvp, precision);
}

extern "C" int tg3_global_scan2d_d(tg3_ctx* c, const float* img, int vdim, int pf, int nImg,
                                   int nR, int nT, const float* dat, const float* ctf,
                                   const float* sigRcp, const double* rot, const double* trans,
                                   const double* pR, const double* pT, double* wC, double* wR,
                                   double* wT, double* baseL, float* dvp, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!img || vdim < 4 || (vdim & 1) || pf < 1) return fail(TG3_ERR_ARG, "bad class image");
    return global_scan(c, nullptr, reinterpret_cast<const float2*>(img), vdim, pf, nImg, nR, nT,
                       dat, ctf, sigRcp, rot, trans, pR, pT, wC, wR, wT, baseL, dvp, precision);
}

// Per-(image, class) weights of a multi-class scan merged over the classes
// to the value the reference's running baseline (kernel_setBaseLine /
// kernel_UpdateW) reaches; the outputs in the ExpectGlobal2D layout.
static int merge_classes(tg3_ctx* c, int n, int nK, int nR, int nT, const double* wCd,
                         const double* wRd, const double* wTd, const double* bd, float* wC,
                         float* wR, float* wT, float* baseL)
{
    TG3_CUDA(launch_merge_classes(n, nK, nR, nT, wCd, wRd, wTd, bd, wC, wR, wT, baseL,
                                  c->stream));
    return TG3_OK;
}

extern "C" int tg3_global_scan2d_classes_d(tg3_ctx* c, const float* imgs, int nK, int vdim,
                                           int pf, int nImg, int nR, int nT, const float* dat,
                                           const float* ctf, const float* sigRcp,
                                           const double* rot, const double* trans,
                                           const double* pR, const double* pT, float* wC,
                                           float* wR, float* wT, float* baseL, int precision)
{
    int st = check_ctx(c);
    if (st) return st;
    if (!imgs || nK < 1 || nK > 6144 || vdim < 4 || (vdim & 1) || pf < 1)
        return fail(TG3_ERR_ARG, "bad class images");
    if (!wC || !wR || !wT || !baseL) return fail(TG3_ERR_ARG, "null device pointer");
    if (nImg <= 0 || nR <= 0 || nT <= 0) return fail(TG3_ERR_ARG, "bad scan shape");
    const size_t blocks = (size_t)nImg * nK;
    Arena ar(c, WS_CLASSES);
    const size_t oC = ar.add(8 * blocks), oR = ar.add(8 * blocks * nR),
                 oT = ar.add(8 * blocks * nT), oB = ar.add(8 * blocks);
    char* b = (char*)ws_get(c, WS_CLASSES, ar.used, &st);
    if (!b) return st;
    double *wCd = (double*)(b + oC), *wRd = (double*)(b + oR), *wTd = (double*)(b + oT),
           *bd = (double*)(b + oB);
    const size_t img = (size_t)vdim * (vdim / 2 + 1);
    st = global_scan(c, nullptr, reinterpret_cast<const float2*>(imgs), vdim, pf, nImg, nR, nT,
                     dat, ctf, sigRcp, rot, trans, pR, pT, wCd, wRd, wTd, bd, nullptr, precision,
                     nK, img);
    if (st) return st;
    return merge_classes(c, nImg, nK, nR, nT, wCd, wRd, wTd, bd, wC, wR, wT, baseL);
}
