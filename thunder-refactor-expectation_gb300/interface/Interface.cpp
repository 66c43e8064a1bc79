/*
 * Interface.cpp -- drop-in definitions of the E-step and insertion entry
 * points of THUNDER's gpu/interface/Interface.h over libtg3.so.
 *
 * The signatures are those of gpu/interface/Interface.h (cited per function);
 * this file replaces the corresponding definitions of the reference's
 * gpu/interface/Interface.cpp.  Entry points outside this path (the
 * reconstruction's Expose* family) keep their reference definitions; ReMask
 * (the images' re-masking ahead of an expectation) and PrepareTF (the
 * accumulators' normalisation and symmetrisation) are defined here.
 *
 * Insertion sums over the hemisphere's ranks inside the call, as the
 * reference's does (ncclAllReduce of F and T over the ranks of `hemi`,
 * gpu/src/cuthunder.cu:4956-5000): every rank inserts its own images on its
 * GPU, then F and T are summed over `hemi` on the host with MPI.  O3D and
 * the counter stay per rank (the reference sums them over the process's own
 * GPUs only).  The kernel follows the reference's build switch:
 * RECONSTRUCTOR_MKB_KERNEL (include/Config.h:95) selects the MKB kernel,
 * otherwise the trilinear one of the reference's GPU insertion.
 *
 * Behaviour kept from the reference: functions return void and a failure
 * prints the library's message and exits the process (the reference's
 * cudaCheckErrors does the same); "device pointers" handed back to the
 * caller are opaque handles the caller only passes back in.
 *
 * Thread safety: the Optimiser calls these from OpenMP threads, holding a
 * per-GPU lock around ExpectLocalRTD / PreI3D / M; the side tables below are
 * guarded by one mutex.
 */
#include "Interface.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "thunder_gb300.h"

static_assert(sizeof(RFLOAT) == sizeof(float),
              "the GB300 library implements the single-precision (RFLOAT = float) interface");

namespace {

std::mutex g_mu;

[[noreturn]] void die(const char* where, int status)
{
    std::fprintf(stderr, "%s: %s (%s)\n", where, tg3_status_string(status), tg3_last_error());
    std::exit(1);
}

inline void ok(const char* where, int status)
{
    if (status != TG3_OK) die(where, status);
}

#ifdef RECONSTRUCTOR_MKB_KERNEL
constexpr int kInsertKernel = TG3_KERNEL_MKB;
#else
constexpr int kInsertKernel = TG3_KERNEL_TRILINEAR;
#endif

// Sum n floats over the ranks of comm in place, in pieces whose counts fit
// an int (MPI_Allreduce_Large does the same, include/Parallel.h:266).
void allreduce_sum(float* buf, size_t n, MPI_Comm& comm, const char* where)
{
    const size_t piece = (size_t)1 << 30;
    for (size_t o = 0; o < n; o += piece) {
        const int cnt = (int)(n - o < piece ? n - o : piece);
        if (MPI_Allreduce(MPI_IN_PLACE, buf + o, cnt, MPI_FLOAT, MPI_SUM, comm) != MPI_SUCCESS) {
            std::fprintf(stderr, "%s: MPI_Allreduce over the hemisphere failed\n", where);
            std::exit(1);
        }
    }
}

// ExpectPreidx: the pixel list, returned to the caller as opaque handles.
struct PixelList {
    std::vector<int> iCol, iRow;
};
std::map<int*, PixelList*> g_pixels;

// ExpectLocalIn: per-GPU image slots (cpyNumL images of npxl pixels).
struct Slots {
    int npxl = 0, n = 0;
    std::vector<Complex> dat;
    std::vector<RFLOAT> ctf, sig, def;
};
std::map<Complex*, Slots*> g_slots;

// ExpectLocalV3D / V2D: the volume (or 2-D class image) behind a
// ManagedArrayTexture.
struct VolState {
    const Complex* host = nullptr;
    int vdim = 0;
    int pf = 0;
    tg3_volume* h = nullptr;
    bool twoD = false;          // bound by ExpectLocalV2D
    int dimSize = 0;            // the class image's element count (2-D)
    tg3_image* img = nullptr;
};

void release(VolState& v)
{
    if (v.h) tg3_volume_destroy(v.h);
    if (v.img) tg3_image_destroy(v.img);
    v.h = nullptr;
    v.img = nullptr;
}
std::map<ManagedArrayTexture*, VolState> g_vols;

// ExpectLocalRTD / PreI3D: the hypothesis set behind a ManagedCalPoint.
struct CalState {
    std::vector<double> rot, trans, oldR, oldT, dpara, oldD;
    int nR = 0, nT = 0, nD = 0;
    int mode = 1;               // ManagedCalPoint mode: 1 for 3-D, 0 for 2-D
    ManagedArrayTexture* mgr = nullptr;
    int idim = 0, npxl = 0;
    const int* iCol = nullptr;
    const int* iRow = nullptr;
    // defocus search (ExpectLocalPreI3D with k1 != 0)
    float k1 = 0, k2 = 0, phaseShift = 0, conT = 0;
    const RFLOAT* freQ = nullptr;
};
std::map<ManagedCalPoint*, CalState> g_cal;

Slots* slots_of(Complex* devdatP)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_slots.find(devdatP);
    if (it == g_slots.end()) die("tg3 Interface: unknown image slots", TG3_ERR_STATE);
    return it->second;
}

const PixelList* pixels_of(int* deviCol)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_pixels.find(deviCol);
    if (it == g_pixels.end()) die("tg3 Interface: unknown pixel list", TG3_ERR_STATE);
    return it->second;
}

}  // namespace

// gpu/interface/Interface.h:16
void getAviDevice(std::vector<int>& gpus)
{
    int ids[64], n = 0;
    ok("getAviDevice", tg3_getAviDevice(ids, 64, &n));
    gpus.assign(ids, ids + (n < 64 ? n : 64));
}

// gpu/interface/Interface.h:18-23
void ExpectPreidx(int gpuIdx, int** deviCol, int** deviRow, int* iCol, int* iRow, int npxl)
{
    (void)gpuIdx;
    PixelList* p = new PixelList();
    p->iCol.assign(iCol, iCol + npxl);
    p->iRow.assign(iRow, iRow + npxl);
    std::lock_guard<std::mutex> lk(g_mu);
    *deviCol = p->iCol.data();
    *deviRow = p->iRow.data();
    g_pixels[*deviCol] = p;
}

// gpu/interface/Interface.h:26-29 (frequencies are used by the defocus
// search only, which this path does not take)
void ExpectPrefre(int gpuIdx, RFLOAT** devfreQ, RFLOAT* freQ, int npxl)
{
    (void)gpuIdx;
    RFLOAT* f = new RFLOAT[npxl];
    std::memcpy(f, freQ, sizeof(RFLOAT) * npxl);
    *devfreQ = f;
}

// gpu/interface/Interface.h:31-38
void ExpectLocalIn(int gpuIdx, Complex** devdatP, RFLOAT** devctfP, RFLOAT** devdefO,
                   RFLOAT** devsigP, int nPxl, int cpyNumL, int searchType)
{
    (void)gpuIdx;
    (void)searchType;
    Slots* s = new Slots();
    s->npxl = nPxl;
    s->n = cpyNumL;
    s->dat.resize((size_t)nPxl * cpyNumL);
    s->ctf.resize((size_t)nPxl * cpyNumL);
    s->sig.resize((size_t)nPxl * cpyNumL);
    s->def.resize((size_t)nPxl * cpyNumL);
    std::lock_guard<std::mutex> lk(g_mu);
    *devdatP = s->dat.data();
    *devctfP = s->ctf.data();
    *devsigP = s->sig.data();
    *devdefO = s->def.data();
    g_slots[*devdatP] = s;
}

// gpu/interface/Interface.h:45-48
void ExpectLocalV3D(int gpuIdx, ManagedArrayTexture* mgr, Complex* volume, int vdim)
{
    (void)gpuIdx;
    std::lock_guard<std::mutex> lk(g_mu);
    VolState& v = g_vols[mgr];
    release(v);
    v.host = volume;
    v.vdim = vdim;
    v.pf = 0;
    v.twoD = false;
}

// gpu/interface/Interface.h:40-43: a class image of dimSize complex values
// (its edge arrives with ExpectLocalPreI2D)
void ExpectLocalV2D(int gpuIdx, ManagedArrayTexture* mgr, Complex* volume, int dimSize)
{
    (void)gpuIdx;
    std::lock_guard<std::mutex> lk(g_mu);
    VolState& v = g_vols[mgr];
    release(v);
    v.host = volume;
    v.vdim = 0;
    v.pf = 0;
    v.twoD = true;
    v.dimSize = dimSize;
}

// gpu/interface/Interface.h:50-62: copy image imgId into slot threadId
void ExpectLocalP(int gpuIdx, Complex* devdatP, RFLOAT* devctfP, RFLOAT* devdefO,
                  RFLOAT* devsigP, Complex* datP, RFLOAT* ctfP, RFLOAT* defO, RFLOAT* sigP,
                  int threadId, int imgId, int npxl, int cSearch)
{
    (void)gpuIdx;
    (void)devctfP;
    (void)devsigP;
    (void)devdefO;
    Slots* s = slots_of(devdatP);
    if (threadId < 0 || threadId >= s->n || npxl != s->npxl) die("ExpectLocalP", TG3_ERR_ARG);
    const size_t src = (size_t)imgId * npxl, dst = (size_t)threadId * npxl;
    std::memcpy(&s->dat[dst], datP + src, sizeof(Complex) * npxl);
    std::memcpy(&s->sig[dst], sigP + src, sizeof(RFLOAT) * npxl);
    if (cSearch) std::memcpy(&s->def[dst], defO + src, sizeof(RFLOAT) * npxl);
    else std::memcpy(&s->ctf[dst], ctfP + src, sizeof(RFLOAT) * npxl);
}

// gpu/interface/Interface.h:64-78
void ExpectLocalHostA(int gpuIdx, RFLOAT** wC, RFLOAT** wR, RFLOAT** wT, RFLOAT** wD,
                      double** oldR, double** oldT, double** oldD, double** trans,
                      double** rot, double** dpara, int mR, int mT, int mD, int cSearch)
{
    (void)gpuIdx;
    (void)cSearch;
    *wC = new RFLOAT[1];
    *wR = new RFLOAT[mR];
    *wT = new RFLOAT[mT];
    *wD = new RFLOAT[mD];
    *oldR = new double[mR];
    *oldT = new double[mT];
    *oldD = new double[mD];
    *trans = new double[mT * 2];
    *rot = new double[mR * 4];
    *dpara = new double[mD];
}

// gpu/interface/Interface.h:80-87: take a copy of the particle's hypotheses
void ExpectLocalRTD(int gpuIdx, ManagedCalPoint* mcp, double* oldR, double* oldT, double* oldD,
                    double* trans, double* rot, double* dpara)
{
    (void)gpuIdx;
    std::lock_guard<std::mutex> lk(g_mu);
    CalState& c = g_cal[mcp];
    // the hypothesis counts are those of ManagedCalPoint::Init (getNR/getNT/getMD);
    // 2-D rotations are (cos, sin) pairs (expectLocalRTD, gpu/src/cuthunder.cu:2683-2697)
    c.nR = mcp->getNR();
    c.nT = mcp->getNT();
    c.nD = mcp->getMD();
    c.mode = mcp->getMode();
    c.rot.assign(rot, rot + (c.mode == 1 ? 4 : 2) * c.nR);
    c.trans.assign(trans, trans + 2 * c.nT);
    c.oldR.assign(oldR, oldR + c.nR);
    c.oldT.assign(oldT, oldT + c.nT);
    if (c.nD > 0 && dpara && oldD) {
        c.dpara.assign(dpara, dpara + c.nD);
        c.oldD.assign(oldD, oldD + c.nD);
    } else {
        c.dpara.clear();
        c.oldD.clear();
    }
}

// gpu/interface/Interface.h:107-123: bind the volume and geometry; the
// projection itself runs inside ExpectLocalM, fused with the scoring
void ExpectLocalPreI3D(int gpuIdx, int datShift, ManagedArrayTexture* mgr, ManagedCalPoint* mcp,
                       RFLOAT* devdefO, RFLOAT* devfreQ, int* deviCol, int* deviRow,
                       RFLOAT phaseShift, RFLOAT conT, RFLOAT k1, RFLOAT k2, int pf, int idim,
                       int vdim, int npxl, int interp)
{
    (void)gpuIdx;
    (void)datShift;
    (void)devdefO;    // the slot's defocus offsets are read in ExpectLocalM
    if (interp != 1) die("ExpectLocalPreI3D: interpolation", TG3_ERR_UNSUPPORTED);
    const PixelList* px = pixels_of(deviCol);
    (void)deviRow;
    std::lock_guard<std::mutex> lk(g_mu);
    VolState& v = g_vols[mgr];
    if (!v.host || v.twoD || v.vdim != vdim) die("ExpectLocalPreI3D: volume not set", TG3_ERR_STATE);
    if (!v.h || v.pf != pf) {
        release(v);
        ok("ExpectLocalPreI3D", tg3_volume_create(&v.h, reinterpret_cast<const float*>(v.host),
                                                  vdim, pf));
        v.pf = pf;
    }
    CalState& c = g_cal[mcp];
    c.mgr = mgr;
    c.idim = idim;
    c.npxl = npxl;
    c.iCol = px->iCol.data();
    c.iRow = px->iRow.data();
    // k1 = k2 = 0 outside the defocus search (src/Optimiser.cpp:2511-2550)
    c.k1 = k1;
    c.k2 = k2;
    c.phaseShift = phaseShift;
    c.conT = conT;
    c.freQ = devfreQ;     // ExpectPrefre's copy of the frequencies
}

// gpu/interface/Interface.h:89-105: the 2-D form (no defocus search)
void ExpectLocalPreI2D(int gpuIdx, int datShift, ManagedArrayTexture* mgr, ManagedCalPoint* mcp,
                       RFLOAT* devdefO, RFLOAT* devfreQ, int* deviCol, int* deviRow,
                       RFLOAT phaseShift, RFLOAT conT, RFLOAT k1, RFLOAT k2, int pf, int idim,
                       int vdim, int npxl, int interp)
{
    (void)gpuIdx;
    (void)datShift;
    (void)devdefO;
    (void)devfreQ;
    (void)phaseShift;
    (void)conT;
    if (interp != 1) die("ExpectLocalPreI2D: interpolation", TG3_ERR_UNSUPPORTED);
    if (k1 != 0 || k2 != 0) die("ExpectLocalPreI2D: 2-D defocus search", TG3_ERR_UNSUPPORTED);
    const PixelList* px = pixels_of(deviCol);
    (void)deviRow;
    std::lock_guard<std::mutex> lk(g_mu);
    VolState& v = g_vols[mgr];
    if (!v.host || !v.twoD || v.dimSize != vdim * (vdim / 2 + 1))
        die("ExpectLocalPreI2D: class image not set", TG3_ERR_STATE);
    if (!v.img || v.pf != pf || v.vdim != vdim) {
        release(v);
        ok("ExpectLocalPreI2D", tg3_image_create(&v.img, reinterpret_cast<const float*>(v.host),
                                                 vdim, pf));
        v.pf = pf;
        v.vdim = vdim;
    }
    CalState& c = g_cal[mcp];
    c.mgr = mgr;
    c.idim = idim;
    c.npxl = npxl;
    c.iCol = px->iCol.data();
    c.iRow = px->iRow.data();
    c.k1 = c.k2 = 0;
}

// gpu/interface/Interface.h:125-139: project, shift, score and return the
// marginal weights of the particle in slot datShift
void ExpectLocalM(int gpuIdx, int datShift, ManagedCalPoint* mcp, Complex* devdatP,
                  RFLOAT* devctfP, RFLOAT* devsigP, RFLOAT* wC, RFLOAT* wR, RFLOAT* wT,
                  RFLOAT* wD, double oldC, int npxl)
{
    (void)gpuIdx;
    (void)devctfP;
    (void)devsigP;
    Slots* s = slots_of(devdatP);
    CalState c;
    tg3_volume* h = nullptr;
    tg3_image* img = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        c = g_cal[mcp];
        h = g_vols[c.mgr].h;
        img = g_vols[c.mgr].twoD ? g_vols[c.mgr].img : nullptr;
    }
    const size_t off = (size_t)datShift * npxl;
    float baseL = 0;
    if (img) {
        if (c.npxl != npxl || c.mode != 0) die("ExpectLocalM: call order", TG3_ERR_STATE);
        ok("ExpectLocalM",
           tg3_ExpectLocal2D(img, reinterpret_cast<const float*>(&s->dat[off]), &s->ctf[off],
                             &s->sig[off], c.iCol, c.iRow, npxl, c.idim, c.rot.data(), c.nR,
                             c.trans.data(), c.nT, c.oldR.data(), c.oldT.data(), oldC, wC, wR,
                             wT, nullptr, &baseL));
        wD[0] = 1;
        return;
    }
    if (!h || c.npxl != npxl) die("ExpectLocalM: call order", TG3_ERR_STATE);
    if (c.k1 != 0 || c.k2 != 0) {
        // defocus search: the slot holds the particle's defocus offsets
        if (c.nD < 1 || (int)c.dpara.size() != c.nD || !c.freQ || s->def.empty())
            die("ExpectLocalM: defocus search state", TG3_ERR_STATE);
        ok("ExpectLocalM",
           tg3_ExpectLocal3D_ctf(h, reinterpret_cast<const float*>(&s->dat[off]), &s->def[off],
                                 c.freQ, c.k1, c.k2, c.phaseShift, c.conT, &s->sig[off], c.iCol,
                                 c.iRow, npxl, c.idim, c.rot.data(), c.nR, c.trans.data(), c.nT,
                                 c.dpara.data(), c.nD, c.oldR.data(), c.oldT.data(),
                                 c.oldD.data(), oldC, wC, wR, wT, wD, nullptr, &baseL));
        return;
    }
    ok("ExpectLocalM",
       tg3_ExpectLocal3D(h, reinterpret_cast<const float*>(&s->dat[off]), &s->ctf[off],
                         &s->sig[off], c.iCol, c.iRow, npxl, c.idim, c.rot.data(), c.nR,
                         c.trans.data(), c.nT, c.oldR.data(), c.oldT.data(), oldC, wC, wR, wT,
                         nullptr, &baseL));
    wD[0] = 1;   // one defocus hypothesis
}

// gpu/interface/Interface.h:141-152
void ExpectLocalHostF(int gpuIdx, RFLOAT** wC, RFLOAT** wR, RFLOAT** wT, RFLOAT** wD,
                      double** oldR, double** oldT, double** oldD, double** trans,
                      double** rot, double** dpara, int cSearch)
{
    (void)gpuIdx;
    (void)cSearch;
    delete[] *wC;
    delete[] *wR;
    delete[] *wT;
    delete[] *wD;
    delete[] *oldR;
    delete[] *oldT;
    delete[] *oldD;
    delete[] *trans;
    delete[] *rot;
    delete[] *dpara;
}

// gpu/interface/Interface.h:154-160
void ExpectLocalFin(int gpuIdx, Complex** devdatP, RFLOAT** devctfP, RFLOAT** devdefO,
                    RFLOAT** devfreQ, RFLOAT** devsigP, int cSearch)
{
    (void)gpuIdx;
    (void)devctfP;
    (void)devdefO;
    (void)devsigP;
    (void)cSearch;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_slots.find(*devdatP);
    if (it != g_slots.end()) {
        delete it->second;
        g_slots.erase(it);
    }
    if (devfreQ && *devfreQ) {
        delete[] *devfreQ;
        *devfreQ = nullptr;
    }
    for (auto& kv : g_vols) release(kv.second);
    g_vols.clear();
    g_cal.clear();
}

// gpu/interface/Interface.h:162-164
void ExpectFreeIdx(int gpuIdx, int** deviCol, int** deviRow)
{
    (void)gpuIdx;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_pixels.find(*deviCol);
    if (it != g_pixels.end()) {
        delete it->second;
        g_pixels.erase(it);
    }
    *deviCol = nullptr;
    *deviRow = nullptr;
}

// gpu/interface/Interface.h:199-208
void ExpectRotran(Complex* traP, double* trans, double* rot, double* rotMat, const int* iCol,
                  const int* iRow, int nR, int nT, int idim, int npxl)
{
    ok("ExpectRotran", tg3_ExpectRotran(reinterpret_cast<float*>(traP), trans, rot, rotMat, iCol,
                                        iRow, nR, nT, idim, npxl));
}

// gpu/interface/Interface.h:210-219
void ExpectProject(Complex* volume, Complex* rotP, double* rotMat, const int* iCol,
                   const int* iRow, int nR, int pf, int interp, int vdim, int npxl)
{
    ok("ExpectProject",
       tg3_ExpectProject(reinterpret_cast<const float*>(volume), reinterpret_cast<float*>(rotP),
                         rotMat, iCol, iRow, nR, pf, interp, vdim, npxl));
}

// gpu/interface/Interface.h:221-237
void ExpectGlobal3D(Complex* rotP, Complex* traP, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
                    RFLOAT* wC, RFLOAT* wR, RFLOAT* wT, double* pR, double* pT, RFLOAT* baseL,
                    int kIdx, int nK, int nR, int nT, int npxl, int imgNum)
{
    ok("ExpectGlobal3D",
       tg3_ExpectGlobal3D(reinterpret_cast<const float*>(rotP), reinterpret_cast<const float*>(traP),
                          reinterpret_cast<const float*>(datP), ctfP, sigRcpP, wC, wR, wT, pR, pT,
                          baseL, kIdx, nK, nR, nT, npxl, imgNum));
}

// gpu/interface/Interface.h:176-197.  vol holds the nK class images
// [vdim][vdim/2 + 1] one after another.
void ExpectGlobal2D(Complex* vol, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP, double* trans,
                    RFLOAT* wC, RFLOAT* wR, RFLOAT* wT, double* pR, double* pT, double* rot,
                    const int* iCol, const int* iRow, int nK, int nR, int nT, int pf, int interp,
                    int idim, int vdim, int npxl, int imgNum)
{
    ok("ExpectGlobal2D",
       tg3_ExpectGlobal2D(reinterpret_cast<const float*>(vol), reinterpret_cast<const float*>(datP),
                          ctfP, sigRcpP, trans, wC, wR, wT, pR, pT, rot, iCol, iRow, nK, nR, nT,
                          pf, interp, idim, vdim, npxl, imgNum));
}

// gpu/interface/Interface.h:239-266.  F2D / T2D hold the nk class
// accumulators [vdim][vdim/2 + 1] one after another.
void InsertI2D(Complex* F2D, RFLOAT* T2D, double* O2D, int* counter, MPI_Comm& hemi,
               MPI_Comm& slav, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP, RFLOAT* w,
               double* offS, int* nC, double* nR, double* nT, double* nD, CTFAttr* ctfaData,
               const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch, int nk, int opf,
               int npxl, int mReco, int idim, int vdim, int imgNum)
{
    (void)slav;
    ok("InsertI2D",
       tg3_InsertI2D(reinterpret_cast<float*>(F2D), T2D, O2D, counter,
                     reinterpret_cast<const float*>(datP), ctfP, sigRcpP, w, offS, nC, nR, nT, nD,
                     reinterpret_cast<const float*>(ctfaData), iCol, iRow, pixelSize,
                     cSearch ? 1 : 0, nk, opf, npxl, mReco, idim, vdim, imgNum));
    // the class accumulators summed over the hemisphere (gpu/src/cuthunder.cu:3913-4017)
    const size_t n = (size_t)nk * vdim * (vdim / 2 + 1);
    allreduce_sum(reinterpret_cast<float*>(F2D), 2 * n, hemi, "InsertI2D");
    allreduce_sum(T2D, n, hemi, "InsertI2D");
}

// gpu/interface/Interface.h:517-522: every image's transform re-masked in place
void ReMask(std::vector<Image>& img, RFLOAT maskRadius, RFLOAT pixelSize, RFLOAT ew, int idim,
            int imgNum)
{
    std::vector<float*> p((size_t)imgNum);
    for (int i = 0; i < imgNum; i++) p[(size_t)i] = reinterpret_cast<float*>(&img[(size_t)i][0]);
    ok("ReMask", tg3_ReMask(p.data(), imgNum, idim, maskRadius, pixelSize, ew));
}

// gpu/interface/Interface.h:320-326: T3D is a complex Volume whose real
// parts hold T; the symmetry matrices come as Eigen dmat33 (column-major,
// Reconstructor::prepareTFG, src/Reconstructor.cpp:1020-1052) and are passed
// on row-major.
void PrepareTF(int gpuIdx, Volume& F3D, Volume& T3D, double* symMat, int nSymmetryElement,
               int maxRadius, int pf)
{
    (void)gpuIdx;
    const size_t n = F3D.sizeFT();
    std::vector<RFLOAT> T(n);
    for (size_t i = 0; i < n; i++) T[i] = REAL(T3D[i]);
    std::vector<double> rowMajor((size_t)9 * (nSymmetryElement > 0 ? nSymmetryElement : 0));
    for (int e = 0; e < nSymmetryElement; e++)
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) rowMajor[9 * e + 3 * a + b] = symMat[9 * e + 3 * b + a];
    ok("PrepareTF", tg3_PrepareTF(reinterpret_cast<float*>(&F3D[0]), T.data(), F3D.nSlcFT(),
                                  rowMajor.data(), nSymmetryElement, maxRadius, pf));
    for (size_t i = 0; i < n; i++) T3D[i] = COMPLEX(T[i], 0);
}

namespace {

// Both InsertFT forms: the library call on T as a real array (the
// reference converts its complex T Volume the same way around the call),
// then the sums over the hemisphere.
void insert_ft(const char* where, Volume& F3D, Volume& T3D, double* O3D, int* counter,
               MPI_Comm& hemi, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
               CTFAttr* ctfaData, double* offS, RFLOAT* w, double* nR, double* nT, double* nD,
               const int* nC, const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch,
               int opf, int npxl, int mReco, int idim, int imgNum)
{
    const size_t n = F3D.sizeFT();
    std::vector<RFLOAT> T(n);
    for (size_t i = 0; i < n; i++) T[i] = REAL(T3D[i]);
    const int vdim = F3D.nSlcFT();
    // CTFAttr (include/Database.h:108-122) is seven RFLOATs in the order the
    // library reads
    static_assert(sizeof(CTFAttr) == 7 * sizeof(RFLOAT), "CTFAttr layout");
    const float* dat = reinterpret_cast<const float*>(datP);
    const float* attr = reinterpret_cast<const float*>(ctfaData);
    float* F = reinterpret_cast<float*>(&F3D[0]);
    if (nC)
        ok(where, tg3_InsertFT_classes(F, T.data(), O3D, counter, dat, ctfP, sigRcpP, attr, offS,
                                       w, nR, nT, nD, nC, iCol, iRow, pixelSize, cSearch ? 1 : 0,
                                       opf, npxl, mReco, idim, vdim, imgNum, kInsertKernel));
    else
        ok(where, tg3_InsertFT(F, T.data(), O3D, counter, dat, ctfP, sigRcpP, attr, offS, w, nR,
                               nT, nD, iCol, iRow, pixelSize, cSearch ? 1 : 0, opf, npxl, mReco,
                               idim, vdim, imgNum, kInsertKernel));
    allreduce_sum(F, 2 * n, hemi, where);
    allreduce_sum(T.data(), n, hemi, where);
    for (size_t i = 0; i < n; i++) T3D[i] = COMPLEX(T[i], 0);
}

}  // namespace

// gpu/interface/Interface.h:294-318 (single-class form).  F3D is complex and
// T3D is a complex Volume whose real parts hold T.
void InsertFT(Volume& F3D, Volume& T3D, double* O3D, int* counter, MPI_Comm& hemi,
              MPI_Comm& slav, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
              CTFAttr* ctfaData, double* offS, RFLOAT* w, double* nR, double* nT, double* nD,
              const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch, int opf,
              int npxl, int mReco, int idim, int dimSize, int imgNum)
{
    (void)slav;
    (void)dimSize;
    insert_ft("InsertFT", F3D, T3D, O3D, counter, hemi, datP, ctfP, sigRcpP, ctfaData, offS, w,
              nR, nT, nD, nullptr, iCol, iRow, pixelSize, cSearch, opf, npxl, mReco, idim,
              imgNum);
}

// gpu/interface/Interface.h:267-292 (multi-class form): the volume of one
// class; nC [imgNum] counts the draws of each image that belong to it.
void InsertFT(Volume& F3D, Volume& T3D, double* O3D, int* counter, MPI_Comm& hemi,
              MPI_Comm& slav, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
              CTFAttr* ctfaData, double* offS, RFLOAT* w, double* nR, double* nT, double* nD,
              int* nC, const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch,
              int opf, int npxl, int mReco, int idim, int dimSize, int imgNum)
{
    (void)slav;
    (void)dimSize;
    insert_ft("InsertFT", F3D, T3D, O3D, counter, hemi, datP, ctfP, sigRcpP, ctfaData, offS, w,
              nR, nT, nD, nC, iCol, iRow, pixelSize, cSearch, opf, npxl, mReco, idim, imgNum);
}
