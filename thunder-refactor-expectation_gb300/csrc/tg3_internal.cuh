// tg3_internal.cuh -- shared declarations of the GB300 E-step library.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <string>
#include <utility>
#include <vector>

#include "thunder_gb300.h"

namespace tg3 {

constexpr int kMaxClasses = 16;
// projection work unit: a lane pair carries kProjU pixels of a chunk of
// kProjChunk (= 128 pairs x kProjU) pixels, for kProjG rotations per CTA
constexpr int kProjU = 4;
constexpr int kProjChunk = 128 * kProjU;
constexpr int kProjG = 8;
// particle-set size held in shared memory by the resampler: 3 doubles and one
// int per entry (8,192 entries = 224 KB of the 227 KB a CTA may hold)
constexpr int kMaxResampleN = 8192;

// ---------------------------------------------------------------- errors --
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define TG3_CUDA(call)                                                   \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return ::tg3::cuda_fail(e_, #call);       \
    } while (0)

#define TG3_LAUNCH_CHECK(what)                                           \
    do {                                                                 \
        cudaError_t e_ = cudaGetLastError();                             \
        if (e_ != cudaSuccess) return ::tg3::cuda_fail(e_, what);        \
    } while (0)

inline size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// ------------------------------------------------- projection volume layout --
// The corner blocks of a volume of edge vdim sit in cubes of 32^3 voxels
// (brick_index in tg3_kernels.cu); cube counts along x (vdim / 2 + 1 stored
// columns) and along y and z.
__host__ __device__ __forceinline__ int cubes_x(int vdim) { return (vdim / 2 + 1 + 31) / 32; }
__host__ __device__ __forceinline__ int cubes_yz(int vdim) { return (vdim + 31) / 32; }

// Per-axis terms of a block's index: block(x, y, z) = tx[x] + ty[y + vdim/2]
// + tz[z + vdim/2] for x in [0, vdim/2], y, z in [-vdim/2, vdim/2), the y and
// z tables absorbing the wrap of negative rows.  tx has vdim/2 + 1 entries,
// ty and tz vdim each; filled by the threads of a CTA (x-stride blockDim.x).
__device__ __forceinline__ void fill_brick_tables(int vdim, int* tx, int* ty, int* tz)
{
    const int nx = vdim / 2 + 1, half = vdim / 2;
    const int nxc = cubes_x(vdim), nyc = cubes_yz(vdim);
    for (int j = threadIdx.x; j < nx; j += blockDim.x)
        tx[j] = (j >> 5) * 32768 + ((j >> 3) & 3) * 512 + (j & 7);
    for (int j = threadIdx.x; j < vdim; j += blockDim.x) {
        const int w = j - half < 0 ? j + half : j - half;
        ty[j] = (w >> 5) * nxc * 32768 + ((w >> 3) & 3) * 2048 + (w & 7) * 8;
        tz[j] = (w >> 5) * nyc * nxc * 32768 + ((w >> 3) & 3) * 8192 + (w & 7) * 64;
    }
}

// ------------------------------------------------------------- workspace --
// Grow-only named device buffers of a context.
enum WsSlot {
    WS_P = 0,        // projections  [rows][Kp] floats
    WS_A,            // shifted, weighted data [nP][nT][Kp]
    WS_D,            // hypothesis-dependent log-likelihood part [nP][nR][nT]
    WS_NRM,          // sum sigRcp ctf^2 |P|^2 per projected row
    WS_PROJ,         // projection scratch: FP32 matrices and norm shares
    WS_FUSED,        // fused launch: particle descriptors, item offsets, counter
    WS_X0,           // sum sigRcp |X|^2 per particle (double)
    WS_PAIRS_TMP,
    WS_H2D,          // staging of host inputs
    WS_D2H,
    WS_BF16,         // split-bf16 operand planes
    WS_MISC,
    WS_INSERT,       // insertion: per-draw pixel grids and rotations
    WS_DEFOCUS,      // defocus search: block priors, block weights
    WS_CLASSES,      // multi-class 2-D scan: per-(image, class) weights
    WS_PREP,         // image preprocessing: statistics, real and transformed images
    WS_RECO,         // reconstruction: T, W, C and the real-space map on the padded grid
    WS_LEARN,        // learned E-step: network outputs, proposals, their weights, fallback lists
    WS_LEARN_IO,     // learned E-step, host-buffer form: staged inputs and outputs
    WS_ORDER,        // bank-row cross term: the particles' visiting order
    WS_RENDER,       // reference rendering: image grid, projections, real images
    WS_SPLITK,       // split-K partial sums of the global search's norm term
    WS_WCHUNK,       // per-chunk weights of a row-split weights launch
    WS_RECO2D,       // 2-D reconstruction: accumulator, staged F / T, image
    WS_COUNT
};

struct Buffer {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct Volume {
    float4* blocks = nullptr;   // volume_block_count(vdim) corner blocks, 4 float4 each
    int vdim = 0;
    int pf = 0;
    size_t bytes = 0;
};

struct Pixels {
    int* iCol = nullptr;
    int* iRow = nullptr;
    int K = 0;
    int Kp = 0;        // floats per padded complex row (multiple of 64)
    int idim = 0;
    double maxRadius = 0;
    int maxAbs = 0;    // max |iCol|, |iRow|
    bool unique = true;
    // pixel of each cell of the half plane [2 maxAbs + 1][maxAbs + 1]
    // (row iRow + maxAbs, column iCol), -1 where none; set when unique
    int* cellPix = nullptr;
    size_t cells = 0;
    unsigned gen = 0;  // upload generation (a bank records the set it was built on)
};

// Projections of one class at a fixed rotation set, made once and gathered
// by index (tg3_ctx_set_bank): FP32 rows [nB][Kp] (complex interleaved,
// zero padded), split-bf16 planes hi, lo [nB][Kp], |P|^2 rows [nB][K].
struct Bank {
    float* f32 = nullptr;
    __nv_bfloat16* hi = nullptr;
    float* abs2 = nullptr;
    double* quat = nullptr;   // the bank's rotations [nB][4]
    int nB = 0, K = 0, Kp = 0;
    unsigned gen = 0;
    size_t bytes = 0;
    // the pose network's embeddings of the clean references at the bank's
    // rotations [nEmb][64], normalised (tg3_ctx_set_references)
    float* emb = nullptr;
    int nEmb = 0;
    // |P|^2 rows [nB][Kq] (zero padded) for the global search's norm term,
    // made on first use from the planes the search reads (abs2qSplit: from
    // hi + lo, else from the FP32 rows; -1: not made)
    float* abs2q = nullptr;
    int abs2qSplit = -1;
};
// The device view of one class's references: embeddings [n][64] and their
// rotations [n][4] (the bank's), for the matching proposals.
struct RefView {
    const float* emb;
    const double* quat;
    int n;
};
// The device view the gather reads, one per class.
struct BankView {
    const float* f32;
    const __nv_bfloat16* hi;
    const __nv_bfloat16* lo;
    const float* abs2;
    int nB;
};

struct InsertAcc {
    float4* acc = nullptr;     // [vdim][vdim][nx] of (F.re, F.im, T, 0)
    int vdim = 0;
    int pf = 0;
    size_t bytes = 0;
    float* tab = nullptr;      // MKB table, nonzero part
    int tabNz = 0;             // last index with a nonzero value
    float tabInvStep = 0;      // n / b
};

}  // namespace tg3

struct tg3_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // host-buffer entries: a second stream for input copies that overlap the
    // first stages, and the event the compute stream waits on (made on first use)
    cudaStream_t copyStream = nullptr;
    cudaEvent_t copyDone = nullptr;
    tg3::Volume vol[tg3::kMaxClasses];
    float4** d_volTable = nullptr;   // device copy of the class -> blocks table
    tg3::Pixels px;                          // the active pixel set (a view)
    tg3::Pixels pxMain;                      // owned: tg3_ctx_set_pixels
    tg3::Pixels pxSlot[tg3::kMaxClasses];    // owned: tg3_ctx_set_pixels_slot
    tg3::InsertAcc ins;
    tg3::Bank bank[tg3::kMaxClasses];        // tg3_ctx_set_bank
    tg3::BankView* d_bankTable = nullptr;    // device copy of the views
    tg3::RefView* d_refTable = nullptr;      // device copy of the reference views
    unsigned pixGen = 0;                     // pixel uploads so far
    tg3::Buffer ws[tg3::WS_COUNT];
    int* d_flag = nullptr;           // device error word
    // tg3_ctx_set_option
    bool fused = false;
    bool insertGather = false;    // TG3_OPT_INSERT_GATHER
    int bankGather = 0;           // TG3_OPT_BANK_GATHER (0, 1 or 2)
    int bankOrder = 1;            // TG3_OPT_BANK_ORDER
    int scanTileN = 0;            // TG3_OPT_SCAN_TILE_N (0: 256)
    int scanPair = 0;             // TG3_OPT_SCAN_PAIR
    int scanBK = 32;              // TG3_OPT_SCAN_BK
    int localBK = 64;             // TG3_OPT_LOCAL_BK
    int projForm = 4;             // TG3_OPT_PROJECT_FORM
    int projGroup = 8;            // TG3_OPT_PROJECT_GROUP
    int bankShape = 3;            // TG3_OPT_BANK_SHAPE
    // per-stage event timing (tg3_ctx_set_timing)
    bool timing = false;
    // inside the learned E-step's fallback: its cross-term launches are
    // recorded as TG3_STAGE_FALLBACK_CROSS and its other inner stages not
    // at all (the bracketing TG3_STAGE_FALLBACK covers them)
    bool fallbackScope = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[TG3_STAGE_COUNT];
    std::vector<cudaEvent_t> eventPool;
    double stageMs[TG3_STAGE_COUNT] = {};
    int stageLaunches[TG3_STAGE_COUNT] = {};
};

namespace tg3 {
// Brackets one stage's launches with events when timing is enabled.
struct StageTimer {
    tg3_ctx* c;
    int stage;
    cudaEvent_t a = nullptr, b = nullptr;
    StageTimer(tg3_ctx* c_, int s);
    ~StageTimer();
};
}  // namespace tg3

struct tg3_volume {
    tg3_ctx* ctx = nullptr;
};

namespace tg3 {

void* ws_get(tg3_ctx* c, WsSlot s, size_t bytes, int* status);

// Bump allocator over one workspace slot (the arrays of one call): add()
// returns 256-byte aligned offsets; ws_get(c, slot, used) then holds them all.
struct Arena {
    tg3_ctx* c;
    WsSlot slot;
    size_t used = 0;
    Arena(tg3_ctx* c_, WsSlot s) : c(c_), slot(s) {}
    size_t add(size_t bytes)
    {
        size_t off = round_up(used, 256);
        used = off + bytes;
        return off;
    }
};

// ---------------------------------------------------------- kernel calls --
// All launchers return cudaError_t of the launch (no synchronisation).
cudaError_t launch_rotmat(const double* quat, int n, double* mat, cudaStream_t st);
cudaError_t launch_translate(const double* trans, int nT, int idim, const int* iCol,
                             const int* iRow, int K, float2* out, int ldo2,
                             cudaStream_t st);
cudaError_t launch_ctf(const float* attr, int nImg, float px, int idim,
                       const int* iCol, const int* iRow, int K, float* out,
                       cudaStream_t st);
// corner blocks the projection volume of edge vdim occupies (64 bytes each)
size_t volume_block_count(int vdim);
cudaError_t launch_volume_blocks(const float2* vol, int vdim, float4* blocks,
                                cudaStream_t st);
// rows: projected rows; a row r belongs to particle r / rowsPerParticle
// (rows a multiple of rowsPerParticle).  Exactly one of quat [rows][4] /
// mat [rows][9] is non-null; nrm is optional.  scratch: device workspace of
// project_scratch_floats(rows, ldo) floats (FP32 matrices, norm shares).
int project_chunks(int ldo);
size_t project_scratch_floats(int rows, int ldo);
cudaError_t launch_project(float4* const* volTable, const int* cls,
                           const float4* vol, int vdim, int pf,
                           const double* quat, const double* mat, int rows,
                           int rowsPerParticle, const int* iCol,
                           const int* iRow, int K, float* out, int ldo,
                           const float* sigRcp, const float* ctf, float* nrm, float* scratch,
                           int* flag, long long splitLo, cudaStream_t st, int form = 4,
                           int group = 8);
// form: 0 a lane pair per pixel (k_project), 1 one lane per pixel
// (k_project_lane, block index from shared tables), 2 one lane per pixel
// with the block index from integer arithmetic, 3 and 4 lane pairs sharing
// loads of whole blocks with the coordinates found once per pixel
// (k_project_xchg; tables, arithmetic); the same samples.  group: the
// rotations a CTA of forms 3 and 4 takes for its pixel chunk (4, 8 or 16).
// Either trans [nP][nT][2] or a shared phase bank [nT][K] complex.
// splitLo != 0: write bf16 hi/lo planes (lo plane splitLo elements after
// the hi plane at `out`) instead of floats; the same for launch_project.
// rows (l nD + d) nT + t; ctf [nP][nD][K] (nD = 1: one CTF per particle)
cudaError_t launch_shift_bank(const float2* dat, const float* ctf,
                              const float* sigRcp, const double* trans,
                              const float2* bank,
                              int nP, int nT, int idim, const int* iCol,
                              const int* iRow, int K, float* out, int ldo,
                              long long splitLo, cudaStream_t st, int nD = 1);
// Defocus search: norms nrm[r][l][d] of the projected rows for each CTF
// (ctf [nP][nD][K], nD <= 16), per-block copies of a particle's priors, and
// the merge of the (particle, defocus) blocks' weights.
cudaError_t launch_norm_defocus(const float* P, long long splitLo, int nP, int nR, int nD, int K,
                                int Kp, const float* sigRcp, const float* ctf, float* nrm,
                                cudaStream_t st);
cudaError_t launch_repeat_rows(const double* src, int rows, int len, int nRep, double* dst,
                               cudaStream_t st);
// 2-D insertion of nDraws draws into per-class accumulators acc
// [nK][vdim][vdim/2 + 1] (F.re, F.im, T, 0); nR, nT [nDraws][2]; nC [nDraws]
cudaError_t launch_insert2d(float4* acc, int vdim, const float2* dat, const float* ctf,
                            int ctfPerDraw, const float* w, const double* offS, const int* nC,
                            const double* nR, const double* nT, const int* iCol, const int* iRow,
                            int K, int pf, int idim, int nDraws, int drawsPerImage, double* O2D,
                            int* counter, cudaStream_t st);
// 2-D projections of a class image [vdim][vdim/2 + 1] at in-plane rotations
// rot [nR][2] (cos, sin): rows out [nR][ldo] (FP32, or split planes)
cudaError_t launch_project2d(const float2* img, int vdim, int pf, const double* rot, int nR,
                             const int* iCol, const int* iRow, int K, float* out, int ldo,
                             long long splitLo, cudaStream_t st);
// CTF attributes [nDraws][7] of insertion draws: the image's, defocus x nD[d]
cudaError_t launch_draw_attr(const float* attr, const double* nD, int nDraws, int drawsPerImage,
                             float* out, cudaStream_t st);
// one particle's CTFs at defocus factors dpara [nD] from per-pixel defocus
// defO and frequency freQ: ctf [nD][K]
cudaError_t launch_ctf_defocus(const float* defO, const float* freQ, const double* dpara, int nD,
                               int K, double k1, double k2, double phaseShift, double conT,
                               float* ctf, cudaStream_t st);
cudaError_t launch_merge_defocus(int nP, int nD, int nR, int nT, const double* wCb,
                                 const double* wRb, const double* wTb, const double* baseb,
                                 const double* pwD, double* wC, double* wR, double* wT,
                                 double* wD, double* base, cudaStream_t st);
cudaError_t launch_x0(const float2* dat, const float* sigRcp, int nP, int K,
                      double* x0, cudaStream_t st);
// C[b][i][j] = alpha * sum_k A[b][i][k] B[b][j][k] + nrm[b][i]   (FP32).
// cGroup > 0: column j is written to group j / cGroup (cGroupStride
// elements apart) at column j % cGroup.
cudaError_t launch_gemm_nt_fp32(const float* A, long long sA, int lda,
                                const float* B, long long sB, int ldb,
                                int M, int N, int Kd, int batch, float* C,
                                long long sC, int ldc, const float* nrm,
                                long long sN, float alpha, cudaStream_t st,
                                int cGroup = 0, long long cGroupStride = 0);
// nrmG (optional) adds a per-(rotation, block) term nrmG[r nrmRS + blk].
// out[i] = sum_b part[b cnt + i], b = 0 .. S-1 in order.
cudaError_t launch_sum_parts(const float* part, int S, size_t cnt, float* out, cudaStream_t st);
cudaError_t launch_weights(const float* D, long long sD, int ldc, int nR,
                           int nT, int G, int nBlocks, const float* nrmG,
                           int nrmRS, const double* x0,
                           const double* pwR, long long sR, const double* pwT,
                           long long sT, const double* pwC, double* wC,
                           double* wR, double* wT, double* base, float* dvp,
                           cudaStream_t st, int threads = 512, int nc = 1,
                           double* chunkTmp = nullptr);
// doubles of chunkTmp launch_weights needs for nBlocks items of nc chunks
inline size_t weights_chunk_doubles(int nBlocks, int nc, int nT)
{
    return (size_t)nBlocks * nc * (2 + (size_t)nT);
}
cudaError_t launch_resample(int nP, int n, const double* u, const double* w,
                            const int* perm, const double* u0,
                            const double* peak, int nOut, int* src,
                            double* wOut, int* top, int* flag,
                            cudaStream_t st,
                            const int* nPer = nullptr);
// k_insert_draws (one thread per draw: parameters into params, 16 floats
// per draw, and the O3D / counter bookkeeping), then k_insert: CTA (share
// of the pixels, draw); draw d uses image d / drawsPerImage.
cudaError_t launch_insert(float4* acc, int vdim, int kernel, const float* tab,
                          int tabNz, float tabInvStep, int nDraws,
                          int drawsPerImage, const float2* dat,
                          const float* ctf, const double* quat,
                          const double* trans, const double* offset,
                          const float* w, const int* iCol, const int* iRow,
                          int K, int pf, int idim, double* O3D, int* counter,
                          float* params, cudaStream_t st, int ctfRows = 0,
                          const int* nC = nullptr);
// MKB insertion by gather: per chunk of draws, k_insert_stage (tiles x
// draws) fills the draws' dense pixel grids from the cell map cellPix,
// k_insert_gather (tiles x draws) adds each slab voxel once.  scratch holds
// insert_draw_bytes(Rg) per draw of a chunk; pixels must be unique.
size_t insert_draw_bytes(int Rg);
cudaError_t launch_insert_gather(float4* acc, int vdim, const float* tab, int tabNz,
                                 float tabInvStep, int nDraws, int drawsPerImage,
                                 const float2* dat, const float* ctf, const double* quat,
                                 const double* trans, const double* offset, const float* w,
                                 const int* cellPix, const int* iCol, const int* iRow, int K,
                                 int pf, int idim, int Rg, float Rp, double* O3D, int* counter,
                                 void* scratch, size_t scratchBytes, cudaStream_t st,
                                 int ctfRows = 0);
// Bank of projections: split planes and |P|^2 rows from the FP32 rows.
cudaError_t launch_bank_planes(const float* f32, int nB, int K, int Kp, __nv_bfloat16* hi,
                               __nv_bfloat16* lo, float* abs2, cudaStream_t st);
// P rows [nP * nR][Kp] (FP32, or hi / lo planes when splitLo != 0) gathered
// from the banks of the particles' classes at idx [nP][nR], and the rows'
// norms sum sigRcp ctf^2 |P|^2.  An index outside the bank sets flag bit 16
// and yields a zero row.
cudaError_t launch_bank_gather(const BankView* table, const int* cls, const int* idx, int nP,
                               int nR, int K, int Kp, const float* sigRcp, const float* ctf,
                               float* P, long long splitLo, float* nrm, int* flag,
                               cudaStream_t st);
// Pose network inference on the tensor cores (tg3_conv_tc.cu).  One layer
// as an implicit GEMM: in NHWC bf16 [n][H][W][Cin] (Cin a multiple of 32),
// w [coutPad][Kpad] bf16 with K = tap * Cin + ci (tap = ky * ks + kx),
// out NHWC bf16 [n][Ho][Wo][Cout] after bias (FP32) and optional ReLU.
struct ConvTcArgs {
    const __nv_bfloat16* in;
    const __nv_bfloat16* w;
    const float* bias;
    __nv_bfloat16* out;
    int n, H, W, Cin, Ho, Wo, Cout, coutPad, ks, stride, pad, Kpad, tmemCols, relu;
    int kSplit;          // K slices (1: no split); > 1 needs partial
    float* partial;      // [kSplit][M][Cout] FP32 sums of the slices
    int* flag;
};
size_t conv_tc_smem(int coutPad);
cudaError_t launch_conv_tc(const ConvTcArgs& a, cudaStream_t st);
// first layer: FP32 images [n][H][H], w [32][9] bf16, out NHWC bf16 [n][H][H][32]
cudaError_t launch_conv1_nhwc(const float* img, const __nv_bfloat16* w, const float* bias, int n,
                              int H, __nv_bfloat16* out, cudaStream_t st);
// output layer: out [n][N] = act [n][K] (bf16) W^T (bf16 [N][K]) + bias
cudaError_t launch_fc_out(const __nv_bfloat16* act, const __nv_bfloat16* w, const float* bias,
                          int n, int K, int N, float* out, cudaStream_t st);
// Shell correlation of two half volumes; sums holds 3 nShell doubles.
cudaError_t launch_fsc(const float2* A, const float2* B, int vdim, int nShell,
                       double* sums, double* fsc, cudaStream_t st);
cudaError_t launch_acc_ratio(const float4* acc, size_t n, float floor_, float2* V,
                             cudaStream_t st);
cudaError_t launch_acc_read(const float4* acc, size_t n, float2* F, float* T,
                            int accumulate, cudaStream_t st);
cudaError_t launch_merge_class(int nImg, int nK, int kIdx, int nR, int nT,
                               const double* wCn, const double* wRn,
                               const double* wTn, const double* basen,
                               float* wC, float* wR, float* wT, float* baseL,
                               cudaStream_t st, int inStride = 1);
// Per-(image, class) weights wCn / basen [nImg][nK], wRn [nImg][nK][nR],
// wTn [nImg][nK][nT] merged over the classes into ExpectGlobal2D's float
// outputs relative to each image's best class (nK <= 6144)
cudaError_t launch_merge_classes(int nImg, int nK, int nR, int nT, const double* wCn,
                                 const double* wRn, const double* wTn, const double* basen,
                                 float* wC, float* wR, float* wT, float* baseL, cudaStream_t st);
// Row norms of a multi-class scan regrouped per (image, class) block:
// out[r][l nK + k] = nrm[(k nR + r) n + l]
cudaError_t launch_nrm_classes(const float* nrm, int nK, int nR, int n, float* out,
                               cudaStream_t st);

// Split-bf16 tensor-core cross term (tcgen05), when available.
// ------------------------------------------- fused projection + scoring --
// One particle of a fused launch: its class, hypothesis counts, first row of
// its rotation matrices and of its shifted-data planes, the offset of its
// sigRcp / ctf values, and the first element of its [nR][nT] likelihoods.
struct FusedParticle {
    int cls;
    int nR, nT;
    int rowOff;
    int transRow;
    int sgOff;
    long long dOff;
};
// A class's pixel set (K pixels; Kp padded floats per row, a multiple of 64).
struct FusedPixels {
    const int* iCol;
    const int* iRow;
    int K, Kp;
};
int fused_items(int nR);                              // work items of one particle
size_t fused_smem_bytes(int vdim, int ntile, int* stages);
cudaError_t launch_fused_uniform_setup(int nP, int nR, int nT, int K, const int* cls,
                                       FusedParticle* part, int* itemOff, cudaStream_t st);
// D as launch_gemm_bf16x3 would write it from k_project's slices (alpha times
// the split-bf16 cross term plus the row norm), for every particle of `part`;
// B: hi plane of the shifted data (rowsB x KpB bf16), lo plane after it;
// pix: host array of kMaxClasses pixel sets; counter: one device int.
cudaError_t launch_fused_bf16x3(float4* const* volTable, int vdim, int pf, const float* mf,
                                const FusedParticle* part, const int* itemOff, int nP,
                                int nItems, const FusedPixels* pix, const float* sigRcp,
                                const float* ctf, const void* B, long long rowsB, int KpB,
                                int maxNT, float* D, float alpha, int* flag, int* counter,
                                cudaStream_t st);
// FP32 rotation matrices [rows][9] from quaternions or FP64 matrices.
cudaError_t launch_rot_f32(const double* quat, const double* mat, int rows, float* mf,
                           cudaStream_t st);

bool bf16x3_available();
// The bank-row cross term (tg3_bank_gemm.cu): C [nP][nR][nT] = alpha x the
// split product of the rows idx [nP][nR] of the particles' class banks with
// the shifted data B (hi plane [nP nT][Kd], then the lo plane), plus the
// rows' norms sum_p sigRcp ctf^2 |P|^2 (compensated FP32).  shape (the
// cp.async form): 0 K blocks of 64 bf16, one CTA an SM; 1 K blocks of 32,
// twice the stages; 2 K blocks of 32, two CTAs an SM; 3 as 0 with 16
// gather warps instead of 8.
cudaError_t launch_gemm_bank_bf16x3(const Bank* banks, unsigned pixGen, const int* idx,
                                    const int* cls, int nP, int nR, const void* B, int nT,
                                    int Kd, int K, const float* sigRcp, const float* ctf,
                                    float* C, float alpha, int* flag, cudaStream_t st,
                                    bool tmaGather = false, int* order = nullptr, int shape = 3);
cudaError_t launch_gemm_nt_bf16x3(const float* A, long long sA, int lda,
                                  const float* B, long long sB, int ldb,
                                  int M, int N, int Kd, int batch, float* C,
                                  long long sC, int ldc, const float* nrm,
                                  long long sN, float alpha, void* scratch,
                                  size_t scratchBytes, int* flag,
                                  cudaStream_t st, int bk = 64);
size_t bf16x3_scratch_bytes(int M, int N, int Kd, int batch);
// General split-bf16 GEMM over `items` (see tg3_tc.cu): A/B point at hi
// planes followed by lo planes of rowsA / rowsB rows of Kd bf16 elements.
cudaError_t launch_gemm_bf16x3(const void* A, long long rowsA, const void* B, long long rowsB,
                               int M, int N, int Kd, int items, int aRowsPerItem,
                               int bRowsPerItem, int nTotal, float* C, long long sC, int ldc,
                               const float* nrm, long long sN, float alpha, int* flag,
                               cudaStream_t st, int cGroup = 0, long long cGroupStride = 0,
                               bool pair = false, int bk = 64);

}  // namespace tg3

namespace tg3 {
// Makes the context's device current; TG3_ERR_ARG for a null context.
int check_ctx(tg3_ctx* c);
// the active pixel set, scaled by pf, fits a volume of vdim with `margin` to spare
int check_geometry(tg3_ctx* c, int vdim, int pf, double margin = 1.0);
// releases the context's preprocessing and reconstruction FFT plans
void prep_release(tg3_ctx* c);
void reco_release(tg3_ctx* c);
// The global scan of nImg images against class `cls`'s projection bank (its
// nB rotations, already projected on the active pixel set) x nT
// translations; outputs as tg3_global_scan_d with nR = nB.
int global_scan_bank(tg3_ctx* c, int cls, int nImg, int nT, const float* dat, const float* ctf,
                     const float* sigRcp, const double* trans, const double* pR,
                     const double* pT, double* wC, double* wR, double* wT, double* baseL,
                     float* dvp, int precision);
// Uploads the device views of the banks (BankView) and of the references
// (RefView); anyBank / anyRef report whether any class has one on the
// active pixel set.
int upload_bank_views(tg3_ctx* c, bool* anyBank, bool* anyRef);
// Matching proposals (tg3_cnn.cu): particle l matches the references of its
// class cls[l] (table[cls[l]]); maxRef bounds every class's reference count.
cudaError_t launch_match_propose_classes(const float* out, int n, const RefView* table,
                                         const int* cls, int maxRef, int nRot, int nTrans,
                                         unsigned long long seed, double* quat, double* trans,
                                         int* idx, cudaStream_t st);
}  // namespace tg3
