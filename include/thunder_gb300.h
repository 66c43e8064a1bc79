/*
 * thunder_gb300.h -- C ABI of the GB300-native THUNDER E-step + insertion
 * library (libtg3.so).
 *
 * Every entry point returns an int status (TG3_OK on success); the message of
 * the last failure on the calling thread is available from tg3_last_error().
 * Plain pointers and sizes only.  Complex numbers are interleaved
 * (re, im) float pairs, the layout of THUNDER's Complex with RFLOAT = float
 * (include/Precision.h:65-99 of the reference).
 *
 * Two layers:
 *  1. Reference-shaped entry points (tg3_Expect*, tg3_InsertFT): host
 *     pointers, the argument meaning and layouts of the functions of
 *     gpu/interface/Interface.h that they replace (cited beside each).  The
 *     drop-in adaptor interface/Interface.cpp in the package maps the
 *     reference's C++ signatures onto them 1:1.
 *  2. Device-resident entry points (tg3_*_d and the context API): device
 *     pointers and a CUDA stream, for callers that keep data in HBM across
 *     calls (the batched particle-filter phase).
 *
 * Geometry conventions (shared by both layers):
 *  - a padded half-FT volume of edge vdim is stored [z][y][x], x in
 *    [0, vdim/2], y and z in [0, vdim) with negative frequencies wrapped
 *    (Volume::iFTHalf, include/Image/Volume.h:566-573);
 *  - rotation matrices are row-major 3x3 doubles; quaternions (w, x, y, z);
 *  - pixel lists iCol/iRow are those of Optimiser::allocPreCalIdx
 *    (src/Optimiser.cpp:7942-7992), K = npxl entries, unpadded units;
 *  - CTF attributes are 7 floats per image in struct CTFAttr order
 *    (voltage, defocusU, defocusV, defocusTheta, Cs, amplitudeContrast,
 *    phaseShift; include/Database.h:108-122).
 */
#ifndef THUNDER_GB300_H
#define THUNDER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TG3_OK = 0,
    TG3_ERR_ARG = 1,       /* bad argument (null pointer, size, layout) */
    TG3_ERR_CUDA = 2,      /* a CUDA runtime call or kernel launch failed */
    TG3_ERR_ALLOC = 3,     /* device or pinned host allocation failed */
    TG3_ERR_STATE = 4,     /* call out of order (e.g. no volume set) */
    TG3_ERR_TIMEOUT = 5,   /* a bounded device-side wait expired */
    TG3_ERR_NUMERIC = 6,   /* non-finite or all-zero weights */
    TG3_ERR_UNSUPPORTED = 7
};

/* Insertion kernels. */
enum { TG3_KERNEL_TRILINEAR = 0, TG3_KERNEL_MKB = 1 };

/* Scoring precision of the likelihood cross term. */
enum { TG3_SCORE_FP32 = 0, TG3_SCORE_BF16X3 = 1 };

const char* tg3_status_string(int status);
const char* tg3_last_error(void);
/* Library version string, e.g. "tg3 1.0 sm_103a". */
const char* tg3_version(void);

/* ------------------------------------------------------------------------
 * Layer 1: reference-shaped entry points (host pointers).
 * --------------------------------------------------------------------- */

/* Replaces getAviDevice(std::vector<int>&), gpu/interface/Interface.h:16.
 * Writes up to `cap` usable device ordinals to gpus; *n gets the count. */
int tg3_getAviDevice(int* gpus, int cap, int* n);

/* Replaces ExpectRotran, gpu/interface/Interface.h:199-208.
 * traP [nT][npxl] complex: exp(-2 pi i (iCol tx + iRow ty) / idim) for the
 * translations trans [nT][2]; rotMat [nR][9] from the quaternions
 * rot [nR][4]. */
int tg3_ExpectRotran(float* traP, const double* trans, const double* rot,
                     double* rotMat, const int* iCol, const int* iRow,
                     int nR, int nT, int idim, int npxl);

/* Replaces ExpectProject, gpu/interface/Interface.h:210-219.
 * rotP [nR][npxl] complex = trilinear samples of volume (edge vdim, padded
 * by pf) at rotMat (iCol pf, iRow pf, 0).  interp must be linear (1). */
int tg3_ExpectProject(const float* volume, float* rotP, const double* rotMat,
                      const int* iCol, const int* iRow, int nR, int pf,
                      int interp, int vdim, int npxl);

/* Replaces ExpectGlobal3D, gpu/interface/Interface.h:221-237.
 * Scores every (image, rotation, translation) of class kIdx of nK and folds
 * the weights into wC [imgNum][nK], wR [imgNum][nK][nR], wT [imgNum][nK][nT]
 * relative to the running per-image baseline baseL [imgNum].  kIdx == 0
 * initialises; kIdx > 0 rescales earlier classes when the baseline rises.
 * datP/ctfP/sigRcpP are image-major [imgNum][npxl]; pR [nR], pT [nT] are the
 * prior weights. */
int tg3_ExpectGlobal3D(const float* rotP, const float* traP, const float* datP,
                       const float* ctfP, const float* sigRcpP, float* wC,
                       float* wR, float* wT, const double* pR, const double* pT,
                       float* baseL, int kIdx, int nK, int nR, int nT, int npxl,
                       int imgNum);

/* Replaces InsertFT (single-class form), gpu/interface/Interface.h:294-318,
 * on one GPU (no hemisphere/slave communicators).  For every image l and
 * draw m < mReco: rotation from the quaternion nR[(l mReco + m) 4 ..],
 * translation nT[(l mReco + m) 2 ..], shift the image by -(t - offS[l]),
 * weight w[l], and grid datP * ctfP * w into F3D and ctfP^2 * w into T3D
 * (edge dimSize = opf idim), with the trilinear kernel (the reference GPU
 * behaviour) or the MKB kernel (radius a = 1.9, alpha = 15, tabulated as in
 * Reconstructor).  iCol/iRow are the reconstructor's padded pixel indices
 * (i opf, Optimiser.cpp:7984-7986), as the reference passes them.  O3D [3]
 * accumulates -R (t - offS, 0), counter the number of inserted draws.  F3D
 * is complex, T3D real, both [dimSize][dimSize][dimSize/2 + 1],
 * accumulated into (not cleared).  Note: dimSize here is the volume edge;
 * the reference's InsertFT passes the voxel count in its dimSize and the
 * edge (F3D.nSlcFT()) to its back end.
 * With cSearch the CTF of every draw is made on the device from the
 * image's CTFAttr (ctfaData [imgNum][7] floats, CTFAttr field order) with
 * defocusU, V scaled by the draw's factor nD [imgNum][mReco] at pixelSize
 * (kernel_CalculateCTF, gpu/src/Kernel.cu:2132-2198) and ctfP is not read;
 * without it ctfP [imgNum][npxl] is.  kernel is TG3_KERNEL_*. */
int tg3_InsertFT(float* F3D, float* T3D, double* O3D, int* counter,
                 const float* datP, const float* ctfP, const float* sigRcpP,
                 const float* ctfaData, const double* offS, const float* w,
                 const double* nR, const double* nT, const double* nD,
                 const int* iCol, const int* iRow, float pixelSize,
                 int cSearch, int opf, int npxl, int mReco, int idim,
                 int dimSize, int imgNum, int kernel);

/* Replaces the multi-class InsertFT, gpu/interface/Interface.h:267-292
 * (gpu/src/cuthunder.cu:4099): as tg3_InsertFT for the volume of one
 * class, with nC [imgNum] the number of image l's draws that belong to it:
 * draw m of image l is inserted, and counted in O3D and counter, only when
 * m < nC[l] (0 <= nC[l] <= mReco; Optimiser::reconstructRef draws each
 * image's classes and passes their counts, src/Optimiser.cpp:6808-6900). */
int tg3_InsertFT_classes(float* F3D, float* T3D, double* O3D, int* counter,
                         const float* datP, const float* ctfP, const float* sigRcpP,
                         const float* ctfaData, const double* offS, const float* w,
                         const double* nR, const double* nT, const double* nD,
                         const int* nC, const int* iCol, const int* iRow, float pixelSize,
                         int cSearch, int opf, int npxl, int mReco, int idim, int dimSize,
                         int imgNum, int kernel);

/* Local particle-filter scoring of one particle, the combined work of
 * ExpectLocalRTD + ExpectLocalPreI3D + ExpectLocalM,
 * gpu/interface/Interface.h:80-139 (no defocus search): project the nR
 * rotations rot [nR][4] of the current volume handle, shift by the nT
 * translations trans [nT][2], score against dat/ctf/sigRcp [npxl] and
 * return wC [1], wR [nR], wT [nT] relative to the best hypothesis, with the
 * prior weights oldR [nR], oldT [nT], oldC.  Optional dvp [nR][nT] (may be
 * NULL) receives the log-likelihoods and baseL the best one. */
typedef struct tg3_volume tg3_volume;
int tg3_volume_create(tg3_volume** vol, const float* volume, int vdim, int pf);
int tg3_volume_destroy(tg3_volume* vol);
int tg3_ExpectLocal3D(tg3_volume* vol, const float* dat, const float* ctf,
                      const float* sigRcp, const int* iCol, const int* iRow,
                      int npxl, int idim, const double* rot, int nR,
                      const double* trans, int nT, const double* oldR,
                      const double* oldT, double oldC, float* wC, float* wR,
                      float* wT, float* dvp, float* baseL);

/* The same for 2-D classification's local phase, the combined work of
 * ExpectLocalV2D + ExpectLocalRTD + ExpectLocalPreI2D + ExpectLocalM
 * (gpu/interface/Interface.h:40-43, 80-105, 125-139): the nR in-plane
 * rotations rot [nR][2] = (cos, sin) of a class image (sampled bilinearly
 * at (c i pf - s j pf, s i pf + c j pf), kernel_Project2DL,
 * gpu/src/Kernel.cu:750-778), otherwise as tg3_ExpectLocal3D.  The class
 * image handle holds img [vdim][vdim/2 + 1] (complex, host at creation),
 * padded by pf. */
typedef struct tg3_image tg3_image;
int tg3_image_create(tg3_image** img, const float* data, int vdim, int pf);
int tg3_image_destroy(tg3_image* img);
int tg3_ExpectLocal2D(tg3_image* img, const float* dat, const float* ctf,
                      const float* sigRcp, const int* iCol, const int* iRow, int npxl,
                      int idim, const double* rot, int nR, const double* trans, int nT,
                      const double* oldR, const double* oldT, double oldC, float* wC,
                      float* wR, float* wT, float* dvp, float* baseL);
/* The same with the defocus search (cSearch; ExpectLocalP / RTD / PreI3D /
 * M of gpu/interface/Interface.h:50-139 with k1 != 0): the particle's CTF
 * for each of its nD defocus factors dpara is made on the device from its
 * per-pixel defocus defO and frequency freQ, k1, k2, phaseShift and the
 * amplitude contrast conT (kernel_CalCTFL, gpu/src/Kernel.cu:481-512);
 * oldD are the particle's defocus weights; wD [nD] the marginal defocus
 * weights; dvp (may be NULL) [nD][nR][nT].  1 <= nD <= 16. */
int tg3_ExpectLocal3D_ctf(tg3_volume* vol, const float* dat, const float* defO,
                          const float* freQ, float k1, float k2, float phaseShift,
                          float conT, const float* sigRcp, const int* iCol,
                          const int* iRow, int npxl, int idim, const double* rot,
                          int nR, const double* trans, int nT, const double* dpara,
                          int nD, const double* oldR, const double* oldT,
                          const double* oldD, double oldC, float* wC, float* wR,
                          float* wT, float* wD, float* dvp, float* baseL);

/* 2-D classification's global search, ExpectGlobal2D
 * (gpu/interface/Interface.h:176-197): imgNum images (datP [imgNum][npxl]
 * complex, ctfP, sigRcpP [imgNum][npxl]) against nK class images vol
 * [nK][vdim][vdim/2 + 1] complex (2-D half transforms, rows in FFT order) at
 * nR in-plane rotations rot [nR][2] = (cos, sin) and nT translations trans
 * [nT][2], priors pR [nR], pT [nT].  Outputs wC [imgNum][nK], wR
 * [imgNum][nK][nR], wT [imgNum][nK][nT], relative to each image's best
 * hypothesis over all classes.  iCol / iRow are the image's pixels (the
 * projection samples (iCol pf, iRow pf) rotated); interp must be 1 (linear).
 * Host pointers; FP32 scoring. */
int tg3_ExpectGlobal2D(const float* vol, const float* datP, const float* ctfP,
                       const float* sigRcpP, const double* trans, float* wC, float* wR,
                       float* wT, const double* pR, const double* pT, const double* rot,
                       const int* iCol, const int* iRow, int nK, int nR, int nT, int pf,
                       int interp, int idim, int vdim, int npxl, int imgNum);

/* 2-D classification's insertion, InsertI2D (gpu/interface/Interface.h:
 * 239-266, without its communicators): draw d = l mReco + m of image l goes
 * into class nC[d] at in-plane rotation nR[d] = (cos, sin) and shift nT[d]
 * (minus offS[l]) with weight w[l]: F2D (complex) and T2D (real), both
 * [nk][vdim][vdim/2 + 1], accumulated into by bilinear interpolation;
 * O2D [nk][2] and counter [nk] added to.  iCol / iRow are the padded
 * indices (i opf); vdim = opf idim.  cSearch: each draw's CTF from its
 * image's CTFAttr (ctfaData [imgNum][7]) with defocus x nD[d], ctfP unread.
 * Host pointers. */
int tg3_InsertI2D(float* F2D, float* T2D, double* O2D, int* counter, const float* datP,
                  const float* ctfP, const float* sigRcpP, const float* w, const double* offS,
                  const int* nC, const double* nR, const double* nT, const double* nD,
                  const float* ctfaData, const int* iCol, const int* iRow, float pixelSize,
                  int cSearch, int nk, int opf, int npxl, int mReco, int idim, int vdim,
                  int imgNum);

/* Particle-filter narrowing + systematic resampling of one axis of nP
 * particles, Particle::keepHalfHeightPeak + Particle::resample(n, pt)
 * (src/Particle.cpp:1935-1973, 1275-1463) with the shuffle permutation and
 * u0 supplied by the caller (the reference draws them from its RNG).
 * u [nP][n] likelihood weights, w [nP][n] prior weights, perm [nP][n],
 * u0 [nP], peak [nP] (<= 0: no narrowing; NaN: derive it as
 * Particle::setPeakFactor(PAR_R) does in 3D).  Outputs src [nP][nOut]
 * (index of each new sample's source), wOut [nP][nOut] (normalised new
 * priors), top [nP] (index of the best sample).  Host pointers. */
int tg3_resample(int nP, int n, const double* u, const double* w,
                 const int* perm, const double* u0, const double* peak,
                 int nOut, int* src, double* wOut, int* top);

/* ------------------------------------------------------------------------
 * Layer 2: device-resident context (device pointers, caller's stream).
 * A context owns a CUDA stream, the projection volume in the paired-corner
 * layout, the insertion accumulator and a grow-only workspace.
 * --------------------------------------------------------------------- */
typedef struct tg3_ctx tg3_ctx;

int tg3_ctx_create(tg3_ctx** ctx, int device);
int tg3_ctx_destroy(tg3_ctx* ctx);
/* The context's CUDA stream (cudaStream_t) as void*. */
void* tg3_ctx_stream(tg3_ctx* ctx);
int tg3_ctx_sync(tg3_ctx* ctx);
/* Bytes of device workspace currently held. */
size_t tg3_ctx_workspace_bytes(tg3_ctx* ctx);

/* Projection volume for class `cls` (0-based, < 16): device or host complex
 * half-FT volume of edge vdim, padding factor pf.  Copied into the
 * context's layout: 64-byte blocks of a voxel's eight trilinear corners,
 * placed in 32^3-voxel cubes (about 8x the bytes of the volume). */
int tg3_ctx_set_volume(tg3_ctx* ctx, int cls, const float* volume, int vdim,
                       int pf, int volume_on_device);

/* Pixel list (host arrays), shared by all later calls: K pixels, image edge
 * idim.  Fails if a rotated pixel could leave the volume. */
int tg3_ctx_set_pixels(tg3_ctx* ctx, const int* iCol, const int* iRow, int K,
                       int idim);

/* Several pixel sets in one context (no counterpart in the reference): each
 * class of a refinement may have its own cutoff, hence its own pixel list.
 * tg3_ctx_set_pixels_slot uploads a list into slot 0..15;
 * tg3_ctx_use_pixels(slot) makes it the context's active set for the calls
 * that follow (-1: the set of tg3_ctx_set_pixels).  Device inputs of those
 * calls hold K values per particle for the active set. */
int tg3_ctx_set_pixels_slot(tg3_ctx* ctx, int slot, const int* iCol, const int* iRow, int K,
                            int idim);
int tg3_ctx_use_pixels(tg3_ctx* ctx, int slot);

/* Batched local phase of nP particles (all device pointers, layouts
 * particle-major): dat [nP][K] complex, ctf, sigRcp [nP][K]; quat
 * [nP][nR][4], trans [nP][nT][2] (double); priors pwR [nP][nR],
 * pwT [nP][nT] (double), pwC [nP] (double); class index per particle cls
 * [nP] (int, may be NULL for class 0).
 * Outputs: wC [nP], wR [nP][nR], wT [nP][nT] (double, relative to
 * baseL), baseL [nP] (double), dvp [nP][nR][nT] (float, may be NULL).
 * precision: TG3_SCORE_FP32 or TG3_SCORE_BF16X3. */
int tg3_local_phase_d(tg3_ctx* ctx, int nP, int nR, int nT,
                      const float* dat, const float* ctf, const float* sigRcp,
                      const double* quat, const double* trans,
                      const double* pwR, const double* pwT, const double* pwC,
                      const int* cls, double* wC, double* wR, double* wT,
                      double* baseL, float* dvp, int precision);

/* Host-buffer form of tg3_local_phase_d: the same arguments in host memory
 * (pinned memory gives asynchronous copies).  Inputs are staged into the
 * context's workspace, outputs copied back; returns after completion. */
int tg3_local_phase(tg3_ctx* ctx, int nP, int nR, int nT, const float* dat,
                    const float* ctf, const float* sigRcp, const double* quat,
                    const double* trans, const double* pwR, const double* pwT,
                    const double* pwC, const int* cls, double* wC, double* wR,
                    double* wT, double* baseL, float* dvp, int precision);

/* Per-stage device timing (CUDA events on the context stream).  When
 * enabled, every stage launch is bracketed by events; tg3_ctx_stage_times
 * synchronises and returns, per stage, the summed milliseconds and the
 * number of launches since the last reset. */
enum {
    TG3_STAGE_PROJECT = 0, TG3_STAGE_SHIFT = 1, TG3_STAGE_CROSS = 2,
    TG3_STAGE_WEIGHTS = 3, TG3_STAGE_RESAMPLE = 4, TG3_STAGE_INSERT = 5,
    TG3_STAGE_FUSED = 6,   /* projection + split-bf16 cross term in one kernel */
    TG3_STAGE_NETWORK = 7, /* learned E-step: network, matching, proposal confidence */
    TG3_STAGE_FALLBACK = 8,/* learned E-step: global search of the fallback particles */
    TG3_STAGE_FALLBACK_CROSS = 9, /* ... of which its cross-term GEMMs */
    TG3_STAGE_NORM = 10,   /* global search: the norm term sum sigRcp ctf^2 |P|^2 per
                              (rotation, image), in and out of the fallback */
    TG3_STAGE_COUNT = 11
};
int tg3_ctx_set_timing(tg3_ctx* ctx, int enable);

/* Context options (no counterpart in the reference).
 * TG3_OPT_FUSED (default 0): 1 makes the split-bf16 local phase gather every
 *   slice straight into the tensor-core operand of one persistent kernel
 *   (projection + cross term fused, no slice bank in HBM); 0 keeps the
 *   two-kernel form (k_project writing the slice bank, then the GEMM), which
 *   is the faster of the two on GB300.
 * TG3_OPT_INSERT_GATHER (default 0): 1 makes MKB insertion gather each voxel
 *   of a slice's slab from its pixels and add it once (one atomic per voxel);
 *   0 scatters every pixel's support voxels with one atomic each (the
 *   reference's loop order), which is the faster of the two on GB300.  Both
 *   give the same sums up to FP32 rounding order; a pixel list holding a pixel
 *   twice always scatters.
 * TG3_OPT_BANK_GATHER (default 0): how the split-bf16 bank-row local phase
 *   (tg3_local_phase_bank_d, the learned E-step's rescoring) reads the
 *   proposed rows.  0: the GEMM's own warps gather its operand tiles from
 *   the bank rows with cp.async and sum the rows' norms from them
 *   (compensated FP32) -- the fastest.  1: copied into a slice buffer, their
 *   norms summed from the bank's |P|^2 rows, then the GEMM.  2: as 0 with the
 *   tiles loaded by TMA gathers.
 * TG3_OPT_BANK_ORDER (default 1): 1 makes forms 0 and 2 above visit the
 *   particles in the order of their first proposed row (class, then bank
 *   row), so that the particles in flight together share bank rows in L2;
 *   batches of more than 8,192 particles keep their own order.  The results
 *   do not depend on it.
 * TG3_OPT_SCAN_TILE_N (default 0 = 256): the column tile (UMMA N, a multiple
 *   of 16 up to 256) of the split-bf16 global scan's cross term; a narrower
 *   tile leaves room for more pipeline stages.  The results do not depend on
 *   it.
 * TG3_OPT_SCAN_PAIR (default 0): 1 runs that cross term on pairs of CTAs
 *   (a thread-block cluster of two on neighbouring row tiles) that share
 *   each column tile: each CTA loads half of it, multicast to both, halving
 *   the bytes the column operand takes from L2.  Same results.
 * TG3_OPT_SCAN_BK (default 32): the K block of that cross term's pipeline
 *   stages, 64 bf16 (128-byte rows, 128-byte swizzle) or 32 (64-byte rows,
 *   64-byte swizzle: half the bytes a stage, twice the stages in flight).
 *   Same products in the same order.
 * TG3_OPT_LOCAL_BK (default 64): the same choice for the split-bf16 local
 *   phase's cross term (tg3_local_phase_d); an uneven-batch plan created
 *   with an autotuned budget tries both and keeps the faster for its
 *   waves.
 * TG3_OPT_PROJECT_FORM (default 4): how the projection extracts samples,
 *   0 with a lane pair per pixel (each lane one slab of the corner block,
 *   joined by a shuffle), 1 with one lane per pixel, 2 with one lane per
 *   pixel and the block index computed instead of looked up, 3 and 4 with
 *   every lane finding its own pixel's block and a lane pair loading both
 *   pixels' blocks together (index looked up, computed).  Same samples.
 * TG3_OPT_BANK_SHAPE (default 3): the pipeline of the bank-row cross term's
 *   cp.async form (TG3_OPT_BANK_GATHER 0): 0 K blocks of 64 bf16 (128-byte
 *   rows) and one CTA an SM, 1 K blocks of 32 (64-byte rows) with twice the
 *   stages, 2 K blocks of 32 with two CTAs an SM, 3 as 0 with 16 gather
 *   warps instead of 8.  Same products in the same order.
 * TG3_OPT_PROJECT_GROUP (default 8): the rotations one CTA of projection
 *   forms 3 and 4 takes for its 512-pixel chunk (4, 8 or 16).  Same
 *   samples. */
enum {
    TG3_OPT_FUSED = 0,
    TG3_OPT_INSERT_GATHER = 1,
    TG3_OPT_BANK_GATHER = 2,
    TG3_OPT_BANK_ORDER = 3,
    TG3_OPT_SCAN_TILE_N = 4,
    TG3_OPT_SCAN_PAIR = 5,
    TG3_OPT_SCAN_BK = 6,
    TG3_OPT_LOCAL_BK = 7,
    TG3_OPT_PROJECT_FORM = 8,
    TG3_OPT_BANK_SHAPE = 9,
    TG3_OPT_PROJECT_GROUP = 10
};
int tg3_ctx_set_option(tg3_ctx* ctx, int option, int value);
int tg3_ctx_stage_times(tg3_ctx* ctx, double* ms, int* launches, int reset);

/* Uneven batches (no single counterpart in the reference: the batching of
 * Optimiser::expectationG's particle loop, src/Optimiser.cpp:2359-2566, for
 * particles whose rotation / translation sets differ in size after
 * Particle::resample, src/Particle.cpp:1275-1463).  One plan covers nP
 * particles of any classes (each class needs a volume and a pixel slot of the
 * same index).  Host arrays cls, nR, nT give every particle's class and set
 * sizes; every other pointer is a device array packed particle after
 * particle: dat (complex), ctf, sigRcp with the K of the particle's class;
 * quat [4], pwR, permR, wR, srcR, wOutR with its nR entries; trans [2], pwT,
 * permT, wT, srcT, wOutT with its nT entries; pwC, u0R, peakR, u0T, peakT,
 * wC, baseL, topR, topT with one entry.  A run computes for every particle
 * what tg3_local_phase_d followed by tg3_resample_d of its rotations and of
 * its translations (nOut = its own set size) computes for it alone.
 * budget: bytes of projection bank per wave, 0 to autotune; use_graph: the
 * run replays one captured CUDA graph.  Runs are asynchronous on the
 * context stream (tg3_ctx_sync reports device-side errors). */
typedef struct tg3_plan tg3_plan;
int tg3_ragged_plan_create(tg3_ctx* ctx, int nP, const int* cls, const int* nR, const int* nT,
                           const float* dat, const float* ctf, const float* sigRcp,
                           const double* quat, const double* trans, const double* pwR,
                           const double* pwT, const double* pwC, const int* permR,
                           const double* u0R, const double* peakR, const int* permT,
                           const double* u0T, const double* peakT, double* wC, double* baseL,
                           double* wR, double* wT, int* srcR, double* wOutR, int* srcT,
                           double* wOutT, int* topR, int* topT, int precision, size_t budget,
                           int use_graph, tg3_plan** plan);
int tg3_ragged_plan_run(tg3_plan* plan);
int tg3_ragged_plan_info(const tg3_plan* plan, int* waves, size_t* budget);
/* The K block of the plan's split-bf16 cross term (64 or 32: TG3_OPT_LOCAL_BK
 * as the autotuner chose it for this batch, or the context's when the plan
 * was given a budget). */
int tg3_ragged_plan_kblock(const tg3_plan* plan, int* bk);
/* The projection's rotations per CTA in the plan (4, 8 or 16:
 * TG3_OPT_PROJECT_GROUP as the autotuner chose it, or the context's when the
 * plan was given a budget). */
int tg3_ragged_plan_project_group(const tg3_plan* plan, int* group);
int tg3_ragged_plan_destroy(tg3_plan* plan);

/* Pose-proposal network (no counterpart in the reference: a learned seed for
 * the particle filter's rotation and translation samples, rescored by the
 * exact likelihood).  Input: images [n][64][64] float (device).  Output
 * [n][68]: 8 components x (6-D rotation a1 a2, raw concentration, logit),
 * shift mean (2), shift log-variance (2).  All kernels are the library's
 * own; weights are used in bf16 (FP32 master copies), accumulation FP32.
 * tg3_cnn_loss: mean negative log-likelihood of the true poses Rstar
 * [n][9] (row-major) and tstar [n][2] (device); with accumulate_grads its
 * gradient is added to the network's gradient buffer, which tg3_cnn_adam
 * applies (learning rate lr) and tg3_cnn_zero_grads clears.
 * tg3_cnn_params copies the parameters to (set = 0) or from (set = 1) the
 * host; tg3_cnn_set_bf16(net, 0) keeps weights in FP32 (gradient checks). */
typedef struct tg3_cnn tg3_cnn;
int tg3_cnn_create(tg3_cnn** net, int device, unsigned long long seed);
int tg3_cnn_destroy(tg3_cnn* net);
size_t tg3_cnn_param_count(const tg3_cnn* net);
int tg3_cnn_params(tg3_cnn* net, float* host, int set);
int tg3_cnn_grads(tg3_cnn* net, float* host);
int tg3_cnn_set_bf16(tg3_cnn* net, int enable);
int tg3_cnn_forward(tg3_cnn* net, const float* img, int n, float* out);
int tg3_cnn_loss(tg3_cnn* net, const float* img, int n, const double* Rstar,
                 const double* tstar, int accumulate_grads, double* loss);
int tg3_cnn_zero_grads(tg3_cnn* net);
int tg3_cnn_adam(tg3_cnn* net, float lr);
/* Hypotheses from network outputs out [n][68] (device): quat [n][nRot][4]
 * (the 8 component rotations, then rotations drawn by the mixture weights,
 * each turned by a rotation vector ~ N(0, I / kappa)) and trans [n][nTrans][2]
 * ~ N(mu, exp(log-variance)), the first the mean; counter-based random
 * numbers from `seed`.  8 <= nRot <= 512, nTrans <= 512; asynchronous on
 * `stream` (a cudaStream_t, NULL for the default stream). */
int tg3_cnn_propose(const float* out, int n, int nRot, int nTrans, unsigned long long seed,
                    double* quat, double* trans, void* stream);

/* Matching mode of the same network: outputs 0..63 are an embedding,
 * compared by cosine with the embeddings of reference projections of the
 * particle's map; outputs 64..67 stay the shift mean and log-variance.
 * tg3_cnn_backward adds to the gradient buffer the gradient of a loss whose
 * derivative with respect to the outputs for images img is dOut [n][68]
 * (device).
 * tg3_cnn_contrastive: symmetric InfoNCE of n particles against their n
 * reference projections (particle i's positive is reference i) on cosine /
 * tau, plus the Gaussian shift loss against tstar [n][2]; writes dL/d
 * outputs for both (dOutP, dOutR) and the mean loss.  1 < n <= 1024.
 * tg3_cnn_embed: normalised embeddings z [n][64] of outputs [n][68].
 * tg3_cnn_match_propose: per particle, the nRot references of highest cosine
 * score (ref [nRef][64] normalised, refQuat [nRef][4]; ties to the lower
 * index) as quaternions and, when idx is not NULL, as indices idx [n][nRot]
 * (rows of a bank made at refQuat), and nTrans translations drawn as
 * tg3_cnn_propose draws them.
 * nRot <= nRef <= 16384, nTrans <= 512; asynchronous on `stream`. */
int tg3_cnn_backward(tg3_cnn* net, const float* img, int n, const float* dOut);
/* Inference forward for proposals: the same network with bf16 activations
 * (bf16 weights, FP32 accumulation), the wide layers as implicit GEMMs on
 * the tensor cores; outputs [n][68] (device) for images [n][64][64]. */
int tg3_cnn_infer(tg3_cnn* net, const float* img, int n, float* out);
int tg3_cnn_contrastive(tg3_cnn* net, const float* outP, const float* outR, int n,
                        const double* tstar, float tau, float* dOutP, float* dOutR,
                        double* loss);
int tg3_cnn_embed(const float* out, int n, float* z, void* stream);
int tg3_cnn_match_propose(const float* out, int n, const float* ref, int nRef,
                          const double* refQuat, int nRot, int nTrans,
                          unsigned long long seed, double* quat, double* trans, int* idx,
                          void* stream);

/* ------------------------------------------------------ learned E-step --
 * The first expectation of a refinement with the pose network's proposals
 * in place of the uniform global search.  It replaces the global search of
 * ExpectGlobal3D (gpu/interface/Interface.h:221; CPU
 * Optimiser::doGlobalSearch, src/Optimiser.cpp:633-1136), which stays the
 * fallback; the network itself has no counterpart in the reference.
 *
 * Set-up per class k (its volume set, the active pixel set made):
 *   tg3_ctx_set_bank(ctx, k, quat, nB)       projections at nB rotations;
 *   tg3_ctx_set_references(ctx, k, emb, nB)  the network's normalised
 *     embeddings [nB][64] (device) of clean references at the same
 *     rotations (tg3_cnn_infer + tg3_cnn_embed of the rendered references).
 *
 * tg3_learned_expect_d, per particle l of class cls[l] (device inputs:
 * images [nP][64][64] the network's input, dat [nP][K] complex, ctf,
 * sigRcp [nP][K], cls [nP], gTrans [nTg][2] the fallback's translation grid):
 *   1. the network's embedding of the image;
 *   2. proposals: the nRot references of class cls[l] of highest cosine
 *      score (ties to the lower index) x nTrans shifts drawn from the
 *      network's shift output (counter-based, from `seed`);
 *   3. every proposal scored by the exact likelihood (as tg3_local_phase_d,
 *      uniform priors), slices read from the class's bank;
 *   4. confidence peak[l] = (max - median) / (1.4826 (MAD + 1e-12)) of the
 *      nRot x nTrans log-likelihoods;
 *   5. particles with peak[l] < peakMin (or not a number) fall back to the
 *      global search over the bank's nB rotations x gTrans (uniform priors),
 *      reusing the bank's projections.
 * Required outputs (device): bestQuat [nP][4] and bestTrans [nP][2], the
 * argmax of the rotation and of the translation marginals of the method
 * the particle used, and baseL [nP] its largest log-likelihood.  Optional
 * (NULL to skip): peak, fellBack [nP]; the proposals' bank rows propIdx
 * [nP][nRot], rotations propQuat [nP][nRot][4], translations propTrans
 * [nP][nTrans][2], marginals propWR [nP][nRot], propWT [nP][nTrans], best
 * log-likelihood propBase [nP] and log-likelihoods propDvp
 * [nP][nRot][nTrans] (less the per-particle constant, as dvp of
 * tg3_local_phase_d).  nTrans, nTg <= 256, nRot x nTrans <= 16384, nRot at
 * most every used class's reference count.  Returns after the work has
 * finished (the fallback's sizes are read on the host).
 *
 * tg3_ExpectLearned3D: the same with every array in host memory (copied in
 * and out on the context's stream; page-locked buffers copy fastest). */
typedef struct tg3_learned_out {
    double* bestQuat;
    double* bestTrans;
    double* baseL;
    float* peak;
    int* fellBack;
    int* propIdx;
    double* propQuat;
    double* propTrans;
    double* propWR;
    double* propWT;
    double* propBase;
    float* propDvp;
} tg3_learned_out;
int tg3_ctx_set_references(tg3_ctx* ctx, int cls, const float* emb, int n);
int tg3_learned_expect_d(tg3_ctx* ctx, tg3_cnn* net, int nP, const float* images,
                         const float* dat, const float* ctf, const float* sigRcp,
                         const int* cls, int nRot, int nTrans, unsigned long long seed,
                         const double* gTrans, int nTg, float peakMin, int precision,
                         const tg3_learned_out* out);
int tg3_ExpectLearned3D(tg3_ctx* ctx, tg3_cnn* net, int nP, const float* images,
                        const float* dat, const float* ctf, const float* sigRcp,
                        const int* cls, int nRot, int nTrans, unsigned long long seed,
                        const double* gTrans, int nTg, float peakMin, int precision,
                        double* bestQuat, double* bestTrans, double* baseL, float* peak,
                        int* fellBack);

/* The global scan of one 2-D class image img [vdim][vdim/2 + 1] complex
 * (device) at in-plane rotations rot [nR][2] = (cos, sin): otherwise as
 * tg3_global_scan_d. */
int tg3_global_scan2d_d(tg3_ctx* ctx, const float* img, int vdim, int pf, int nImg, int nR,
                        int nT, const float* dat, const float* ctf, const float* sigRcp,
                        const double* rot, const double* trans, const double* pR,
                        const double* pT, double* wC, double* wR, double* wT, double* baseL,
                        float* dvp, int precision);

/* ----------------------------------------------------------- input data --
 * Image preprocessing (Optimiser::initImg, src/Optimiser.cpp:4600-4760, and
 * allocPreCal, :7995-8030): nImg real-space images img [nImg][N][N]
 * (device, file order, x fastest) to the complex pixel data dat [nImg][K]
 * of the context's pixel set (made for idim = N).  Per image: background
 * (i^2 + j^2 > r^2 about pixel (N/2, N/2), r = maskRadiusPx) mean and
 * standard deviation subtracted and divided; with mask, the raised-cosine
 * soft mask of edge 6 pixels to 0 (zeroMask); scaled by 1 / stdN (stdN > 0
 * given, else the batch mean of the normalised background deviations);
 * unnormalised forward transform with the centre at index 0; the pixels
 * gathered.  stats (device, may be NULL): [nImg][3] float background mean,
 * deviation, and normalised deviation. */
int tg3_prepare_images_d(tg3_ctx* ctx, const float* img, int nImg, int N, float maskRadiusPx,
                         int mask, float stdN, float* dat, float* stats);

/* Re-masking of the particle images (Optimiser::reMaskImg,
 * src/Optimiser.cpp:6053-6111; on the GPU reMask, gpu/src/cuthunder.cu:
 * 9384-9560): every image's half transform [N][N/2 + 1] (complex, its centre
 * at index 0) to real space by the normalised inverse transform, times the
 * soft mask of radius maskRadiusPx and edge edgeWidth pixels about the
 * centre (1 inside, 0.5 + 0.5 cos((u - r) / ew pi) on the edge, 0 beyond),
 * back by the unnormalised forward transform.
 * tg3_remask_d: imgFT and out [nImg][N][N/2 + 1] on the device (out may be
 * imgFT); asynchronous on the context's stream.
 * tg3_ReMask replaces ReMask (gpu/interface/Interface.h:517-522): the
 * images are nImg host arrays of idim (idim/2 + 1) complex values,
 * re-masked in place with radius maskRadius / pixelSize (the reference's
 * EDGE_WIDTH_RL is 6); returns when they are written back. */
int tg3_remask_d(tg3_ctx* ctx, const float* imgFT, int nImg, int N, float maskRadiusPx,
                 float edgeWidth, float* out);
int tg3_ReMask(float* const* images, int nImg, int idim, float maskRadius, float pixelSize,
               float ew);

/* The accumulators prepared for reconstruction, as PrepareTF does on the GPU
 * (gpu/src/cuthunder.cu:6160-6400; the CPU path's prepareTF with the
 * normalisation in allReduceT, src/Reconstructor.cpp:1056-1090,
 * 2453-2480): with normalise, F and T scaled by 1 / T at the origin; then
 * both symmetrised -- the volume plus, for every symmetry element R, the
 * volume sampled trilinearly at R v (Friedel mates conjugated) for
 * |R v| < maxRadius pf + 1 (SYMMETRIZE_FT, include/Geometry/
 * Transformation.h:170-196) -- and T floored at 1e-25.  symMat [nSym][9]
 * row-major, the elements other than the identity (nSym <= 64; 0: no
 * symmetrisation).  Asynchronous on the context's stream.
 * tg3_PrepareTF replaces PrepareTF (gpu/interface/Interface.h:320-326) on
 * host arrays: F3D complex and T3D real [vdim][vdim][vdim/2 + 1], replaced
 * in place (normalised and symmetrised); returns when they are written. */
int tg3_ctx_prepare_tf_d(tg3_ctx* ctx, const double* symMat, int nSym, int maxRadius,
                         int normalise);
int tg3_PrepareTF(float* F3D, float* T3D, int vdim, const double* symMat, int nSym,
                  int maxRadius, int pf);

/* The insertion accumulator set to F (complex) and T (real), device arrays
 * [vdim][vdim][vdim/2 + 1] -- e.g. the sums over ranks or half maps that
 * the reference all-reduces before reconstructing (allReduceF / T). */
int tg3_ctx_insert_load_d(tg3_ctx* ctx, const float* F, const float* T);

/* Reconstruction of the map from the context's insertion accumulators
 * (Reconstructor::reconstruct, src/Reconstructor.cpp:1129-1790; 3-D, no
 * symmetry): Wiener filter of T from the FSC per unpadded shell (fsc [nFsc];
 * NULL: none), joined half maps when joinHalf; with gridCorr the balancing of
 * W against the MKB kernel (a, alpha) for up to 30 rounds (rounds returns
 * how many ran; may be NULL), else W = 1 / T; the inverse transform of F W
 * inside maxRadius (unpadded pixels); the central N^3 (N = vdim / pf),
 * divided by the insertion kernel's real-space transform (kernel
 * TG3_KERNEL_TRILINEAR or TG3_KERNEL_MKB).  vol: device float [N][N][N],
 * centred (coordinate i at index i + N/2). */
int tg3_ctx_reconstruct_d(tg3_ctx* ctx, const double* fsc, int nFsc, int joinHalf, int maxRadius,
                          int gridCorr, int kernel, float a, float alpha, float* vol, int* rounds);
/* 2-D reconstruction (Reconstructor::reconstruct(Image&) in MODE_2D,
 * src/Reconstructor.cpp:1093-1103 and its _T2D / _W2D / _C2D branches): the
 * same chain as tg3_ctx_reconstruct_d on one class's 2-D accumulators,
 * host buffers: F2D complex and T2D real [vdim][vdim/2 + 1] (the summed
 * InsertI2D accumulators), img [N][N] out (N = vdim / pf, centred:
 * coordinate i at index i + N/2).  The inverse transform's normalisation
 * is 1 / vdim^2. */
int tg3_Reconstruct2D(const float* F2D, const float* T2D, int vdim, int pf,
                      const double* fsc, int nFsc, int joinHalf, int maxRadius,
                      int gridCorr, int kernel, float a, float alpha, float* img,
                      int* rounds);
/* Reconstructor::symmetrizeO (src/Reconstructor.cpp, prepareO under
 * RECONSTRUCTOR_SYMMETRIZE_DURING_RECONSTRUCT): O3D += sum over the symmetry
 * elements symMat [nSym][9] (row-major, the identity excluded) of R O3D,
 * counter *= 1 + nSym -- the offsets' share of the symmetrisation whose F and
 * T share is tg3_PrepareTF.  Host arithmetic, no device. */
int tg3_SymmetrizeO(double* O3D, int* counter, const double* symMat, int nSym);

/* Noise spectrum sigma^2 from the images at their best poses
 * (Optimiser::allReduceSigma, src/Optimiser.cpp:6355-6630): the active pixel
 * set must hold the shells u = rint(|k|) < rSig of the half transform (i in
 * [0, N/2], every row; powerSpectrum, src/Functions/Spectrum.cpp:161-190).
 * Per image (device arrays): masked and unmasked data datM / datN [nImg][K]
 * complex, ctf [nImg][K], rotMat [nImg][9], trans [nImg][2], offset
 * [nImg][2] (may be NULL), group [nImg] (1-based; read when byGroup).  The
 * class-`cls` volume gives the model.  Out (device, double): sig and
 * sigRcp = -0.5 / sig, [nGroup][rSig]; without byGroup every group gets the
 * pooled spectrum.  maskRadius and pixelSize in Angstrom set alpha =
 * sqrt(pi (maskRadius / (N pixelSize))^2). */
int tg3_sigma_d(tg3_ctx* ctx, int cls, int nImg, const float* datM, const float* datN,
                const float* ctf, const double* rotMat, const double* trans, const double* offset,
                const int* group, int nGroup, int byGroup, int rSig, float maskRadius,
                float pixelSize, double* sig, double* sigRcp);

/* MRC stacks (src/Image/ImageFile.cpp): header fields, and sections
 * [first, first + count) as float32 in file order (modes 0, 1, 2, 6).
 * pixelSize (may be NULL) = cella[0] / mx.  Writing: float32 (mode 2) with
 * the header of ImageFile::fillMRCHeader; volume != 0 scales the z cell by
 * the pixel size.  Host pointers. */
int tg3_mrc_info(const char* path, int* nx, int* ny, int* nz, int* mode, float* pixelSize);
int tg3_mrc_read(const char* path, int first, int count, float* out);
int tg3_mrc_write(const char* path, const float* data, int nx, int ny, int nz, float pixelSize,
                  int volume);

/* .thu particle databases (src/Database.cpp; include/Database.h columns
 * THU_VOLTAGE = 0 ... THU_SCORE = 26): tg3_thu_count gives the particle
 * (non-blank line) count; tg3_thu_read fills cols [n][27] (double; the two
 * path columns 7 and 8 hold NaN) and the particle and micrograph paths as n
 * NUL-terminated strings of `stride` bytes (either may be NULL).
 * tg3_thu_write writes Optimiser::saveDatabase's format (src/Optimiser.cpp:
 * 8221-8262): %18.9f reals, %6d group and class ids. */
int tg3_thu_count(const char* path, int* n);
int tg3_thu_read(const char* path, int n, double* cols, char* paths, char* micrographs,
                 int stride);
int tg3_thu_write(const char* path, int n, const double* cols, const char* paths,
                  const char* micrographs, int stride);

/* 2-D classification's global scan of nImg images against nK class images
 * imgs (device, complex [nK][vdim][vdim/2 + 1]) at nR in-plane rotations
 * rot [nR][2] = (cos, sin) x nT translations, every class in one pass (one
 * shifted-data bank, one cross-term GEMM over all classes' rotations), the
 * classes merged in order with the reference's running baseline, as
 * ExpectGlobal2D returns them: wC [nImg][nK], wR [nImg][nK][nR],
 * wT [nImg][nK][nT], baseL [nImg] (float, device). */
int tg3_global_scan2d_classes_d(tg3_ctx* ctx, const float* imgs, int nK, int vdim, int pf,
                                int nImg, int nR, int nT, const float* dat, const float* ctf,
                                const float* sigRcp, const double* rot, const double* trans,
                                const double* pR, const double* pT, float* wC, float* wR,
                                float* wT, float* baseL, int precision);

/* Global scan of nImg images over one shared set of nR rotations and nT
 * translations, for the context's class-`cls` volume: the scan of
 * Optimiser::doGlobalSearch (src/Optimiser.cpp:759-899), the work of
 * ExpectProject + ExpectGlobal3D kept on the device.  rotMat [nR][9] and
 * trans [nT][2] (double), dat [nImg][K] complex, ctf/sigRcp [nImg][K],
 * priors pR [nR], pT [nT].  Outputs per image, relative to its best
 * hypothesis: wC [nImg], wR [nImg][nR], wT [nImg][nT], baseL [nImg]
 * (double); dvp [nImg][nR][nT] (float, may be NULL). */
int tg3_global_scan_d(tg3_ctx* ctx, int cls, int nImg, int nR, int nT,
                      const float* dat, const float* ctf, const float* sigRcp,
                      const double* rotMat, const double* trans,
                      const double* pR, const double* pT, double* wC,
                      double* wR, double* wT, double* baseL, float* dvp,
                      int precision);

/* Local phase with a defocus search (Optimiser::updateSP with
 * SEARCH_TYPE_CTF, src/Optimiser.cpp:1139-1436; the GPU path of
 * ExpectLocalPreI3D / ExpectLocalM with cSearch, gpu/interface/Interface.h
 * :107-140): every particle's nR rotations x nT translations x nD defocus
 * hypotheses, hypothesis d scored with the CTF ctfD [nP][nD][K] (device;
 * the particle's CTF at defocus scaled by its d-th factor, e.g. from
 * tg3_ctf_d with defocusU, V x d).  pwD [nP][nD] are the defocus weights of
 * the particles; outputs as tg3_local_phase_d plus wD [nP][nD], all relative
 * to each particle's best hypothesis; dvp (may be NULL) [nP][nD][nR][nT].
 * 1 <= nD <= 16; the split-bf16 path needs nD nT <= 256. */
int tg3_local_phase_ctf_d(tg3_ctx* ctx, int nP, int nR, int nT, int nD, const float* dat,
                          const float* ctfD, const float* sigRcp, const double* quat,
                          const double* trans, const double* pwR, const double* pwT,
                          const double* pwD, const double* pwC, const int* cls, double* wC,
                          double* wR, double* wT, double* wD, double* baseL, float* dvp,
                          int precision);

/* Projection banks (no single counterpart in the reference: the global
 * search's projections, ExpectProject, src/Optimiser.cpp:759-785, kept for
 * reuse).  tg3_ctx_set_bank projects the class-`cls` volume at nB rotations
 * quat [nB][4] (device, double) over the active pixel set, once.
 * tg3_local_phase_bank_d is tg3_local_phase_d with every particle's nR
 * rotations given as rows bankIdx [nP][nR] (device int) of its class's bank
 * instead of quaternions: the same likelihoods, weights and outputs, without
 * projecting.  A bank serves while its pixel set is the active one; an index
 * outside its class's bank, or into a bank built on another pixel set, is
 * reported at the next synchronising call. */
int tg3_ctx_set_bank(tg3_ctx* ctx, int cls, const double* quat, int nB);
int tg3_local_phase_bank_d(tg3_ctx* ctx, int nP, int nR, int nT, const float* dat,
                           const float* ctf, const float* sigRcp, const int* bankIdx,
                           const double* trans, const double* pwR, const double* pwT,
                           const double* pwC, const int* cls, double* wC, double* wR,
                           double* wT, double* baseL, float* dvp, int precision);

/* Device form of tg3_resample (all pointers device memory, stream of ctx). */
int tg3_resample_d(tg3_ctx* ctx, int nP, int n, const double* u,
                   const double* w, const int* perm, const double* u0,
                   const double* peak, int nOut, int* src, double* wOut,
                   int* top);

/* Insertion accumulator: edge vdim (= pf idim), cleared to zero. */
int tg3_ctx_insert_begin(tg3_ctx* ctx, int vdim, int pf);
/* Insert nP particles' draws (device pointers): dat [nP][K] complex,
 * ctf [nP][K], quat [nP][4], trans [nP][2], offset [nP][2] (double),
 * w [nP] (float); kernel TG3_KERNEL_*.  O3D (device double[3]) and counter
 * (device int) may be NULL. */
int tg3_insert_d(tg3_ctx* ctx, int nP, const float* dat, const float* ctf,
                 const double* quat, const double* trans, const double* offset,
                 const float* w, int kernel, double* O3D, int* counter);
/* Read the accumulator into separate F (complex) and T (real) device
 * arrays of [vdim][vdim][vdim/2+1] entries, adding to their contents
 * when accumulate != 0. */
int tg3_ctx_insert_read_d(tg3_ctx* ctx, float* F, float* T, int accumulate);
/* The inserted slices' average V = F / T (complex, [vdim][vdim][vdim/2+1])
 * where T > floor, 0 elsewhere.  The normalisation that precedes the
 * reference's reconstruction (Reconstructor, src/Reconstructor.cpp:1056-2713)
 * without its W balancing or gridding correction. */
int tg3_ctx_insert_ratio_d(tg3_ctx* ctx, float* V, float floor);

/* Fourier shell correlation of two complex half volumes A, B
 * [vdim][vdim][vdim/2+1] (device): fsc[u] for shells u = rint(|k|) <
 * nShell, 0 for an empty shell (FSC, src/Functions/Spectrum.cpp:302-329).
 * scratch: device double[3 nShell]; nShell <= 8533. */
int tg3_fsc_d(const float* A, const float* B, int vdim, int nShell, double* fsc,
              double* scratch, void* stream);

/* ------------------------------------------------------------------------
 * Allocation-free local scoring.  No counterpart in the reference.
 *
 * For callers that cannot let a library allocate device memory: an
 * application that has given the GPU's memory to its own pool allocator, or
 * one that scores particles from many host threads at once, where every
 * cudaMalloc / cudaFree would synchronise the device and stall the other
 * threads.  It computes what tg3_local_phase_d computes for one particle on
 * the FP32 path, with its scratch in a fixed device array that belongs to the
 * library image (tg3_noalloc_scratch_bytes() bytes, 64 MiB, held by every GPU
 * that loads the library until the process exits).  It calls no allocator.
 *
 * All pointers are device memory: volume is the plain complex half-FT volume
 * [vdim][vdim][vdim/2 + 1] (padding factor pf); iCol/iRow the K unpadded
 * pixel indices of an image of edge idim; dat [K] complex, ctf, sigRcp [K];
 * quat [nR][4], trans [nT][2]; priors pwR [nR], pwT [nT], pwC [1] (NULL for
 * 1).  Outputs as tg3_local_phase_d with nP = 1; dvp may be NULL.
 *
 * Limit: 256 + 4 ((nR + nT) Kp + nR nT + nR) + 512 bytes (rounded up to
 * 256-byte pieces) must fit the scratch, Kp = 2K rounded up to 64; larger
 * sets are rejected with TG3_ERR_ARG.  The call returns after the work has
 * finished on `stream` (cudaStream_t, NULL for the legacy stream): it reads
 * its error word back with a copy on that stream and synchronises that
 * stream only.  The first call on a device looks up the scratch array's
 * device address (cudaGetSymbolAddress) with that device current, and so
 * does the first call after the device's context is re-created (after
 * cudaDeviceReset); make that first call before any stream capture.  Every call shares the one array: calls that
 * may overlap on the GPU (other streams, unsynchronised host threads) race
 * and must not be issued.  Each call writes all the scratch it reads, so no
 * clearing is needed between calls. */
size_t tg3_noalloc_scratch_bytes(void);
int tg3_local_phase_noalloc(const float* volume, int vdim, int pf,
                            const int* iCol, const int* iRow, int K, int idim,
                            const float* dat, const float* ctf,
                            const float* sigRcp, const double* quat, int nR,
                            const double* trans, int nT, const double* pwR,
                            const double* pwT, const double* pwC, double* wC,
                            double* wR, double* wT, double* baseL, float* dvp,
                            void* stream);

/* ------------------------------------------------------------------------
 * Kernel-level device entry points (device pointers, explicit stream).
 * --------------------------------------------------------------------- */
/* rotMat [n][9] (double, row-major) from quat [n][4]. */
int tg3_rotmat_d(const double* quat, int n, double* rotMat, void* stream);
/* out [nT][K] complex phase-shift bank (see tg3_ExpectRotran). */
int tg3_translate_d(const double* trans, int nT, int idim, const int* iCol,
                    const int* iRow, int K, float* out, void* stream);
/* out [nImg][K] CTF values for attr [nImg][7] (CTF(), src/CTF.cpp:98-145). */
int tg3_ctf_d(const float* attr, int nImg, float pixelSize, int idim,
              const int* iCol, const int* iRow, int K, float* out,
              void* stream);
/* out [nR][K] complex projections of the context's class-`cls` volume at
 * rotMat [nR][9] (double). */
int tg3_project_d(tg3_ctx* ctx, int cls, const double* rotMat, int nR,
                  float* out);
/* The learned E-step's reference images (no counterpart in the reference):
 * out [n][img][img] float, the class-`cls` volume projected at rotMat [n][9]
 * (double) over the img x img rfft grid of the volume's own frequencies
 * (columns 0 .. img/2, rows -img/2 .. img/2 - 1, times pf), taken to real
 * space (cuFFT C2R), centred (index 0 in the middle), minus its mean and
 * over its unbiased standard deviation -- the particle images' form at the
 * network's input.  img even, >= 8; the grid must lie inside the volume.
 * Leaves the context's pixel set alone. */
int tg3_ctx_render_references_d(tg3_ctx* ctx, int cls, const double* rotMat,
                                int n, int img, float* out);

#ifdef __cplusplus
}
#endif

#endif /* THUNDER_GB300_H */
