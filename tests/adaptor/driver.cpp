/*
 * Runs the drop-in adaptor (interface/Interface.cpp over libtg3.so) through
 * the reference's own call sequences and writes what the caller receives.
 * TEST INFRASTRUCTURE: built and run by tests/test_gpu_adaptor.py.
 *
 *   driver <case directory> <fake hemisphere ranks>
 *
 * Local expectation, per image, as Optimiser::expectationG drives it
 * (src/Optimiser.cpp:2212-2566): ExpectPreidx, ExpectLocalIn, ExpectLocalV3D
 * once; per image ExpectLocalP into a slot, ExpectLocalHostA,
 * ManagedCalPoint::Init, ExpectLocalRTD, ExpectLocalPreI3D, ExpectLocalM,
 * ExpectLocalHostF; then ExpectLocalFin and ExpectFreeIdx.  Then the same in
 * 2-D mode (ExpectLocalV2D, ExpectLocalPreI2D, in-plane rotations).  Insertion as
 * Reconstructor::insertI (src/Reconstructor.cpp:867-1000): the single-class
 * InsertFT, then the multi-class one with per-image draw counts, each into
 * zeroed volumes with O3D and the counter starting at zero.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "Interface.h"

static int g_fake_ranks = 1;
static long long g_reduced = 0;

extern "C" int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type,
                             MPI_Op op, MPI_Comm comm)
{
    (void)comm;
    if (send != MPI_IN_PLACE || type != MPI_FLOAT || op != MPI_SUM) return 1;
    float* v = static_cast<float*>(recv);
    for (int i = 0; i < count; i++) v[i] *= (float)g_fake_ranks;
    g_reduced += count;
    return MPI_SUCCESS;
}

template <class T>
static std::vector<T> load(const std::string& dir, const char* name, size_t n)
{
    std::vector<T> v(n);
    FILE* f = std::fopen((dir + "/" + name).c_str(), "rb");
    if (!f || std::fread(v.data(), sizeof(T), n, f) != n) {
        std::fprintf(stderr, "driver: cannot read %s\n", name);
        std::exit(2);
    }
    std::fclose(f);
    return v;
}

template <class T>
static void save(const std::string& dir, const char* name, const T* p, size_t n)
{
    FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
    if (!f || std::fwrite(p, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "driver: cannot write %s\n", name);
        std::exit(2);
    }
    std::fclose(f);
}

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    const std::string dir = argv[1];
    g_fake_ranks = std::atoi(argv[2]);
    int box, pf, npxl, nP, nR, nT, mReco;
    {
        FILE* f = std::fopen((dir + "/meta.txt").c_str(), "r");
        if (!f || std::fscanf(f, "%d %d %d %d %d %d %d", &box, &pf, &npxl, &nP, &nR, &nT,
                              &mReco) != 7)
            return 2;
        std::fclose(f);
    }
    const int vdim = box * pf;
    const size_t nvox = (size_t)vdim * vdim * (vdim / 2 + 1);
    auto vol = load<Complex>(dir, "vol.bin", nvox);
    auto iCol = load<int>(dir, "icol.bin", npxl);
    auto iRow = load<int>(dir, "irow.bin", npxl);
    auto dat = load<Complex>(dir, "dat.bin", (size_t)nP * npxl);
    auto ctf = load<RFLOAT>(dir, "ctf.bin", (size_t)nP * npxl);
    auto sig = load<RFLOAT>(dir, "sig.bin", (size_t)nP * npxl);
    auto rot = load<double>(dir, "rot.bin", (size_t)nP * nR * 4);
    auto trs = load<double>(dir, "trans.bin", (size_t)nP * nT * 2);
    auto oR = load<double>(dir, "oldR.bin", (size_t)nP * nR);
    auto oT = load<double>(dir, "oldT.bin", (size_t)nP * nT);

    // ---------------------------------------------------- local expectation
    const int gpu = 0, slots = 2;
    int *deviCol = nullptr, *deviRow = nullptr;
    ExpectPreidx(gpu, &deviCol, &deviRow, iCol.data(), iRow.data(), npxl);
    Complex* devdatP = nullptr;
    RFLOAT *devctfP = nullptr, *devdefO = nullptr, *devsigP = nullptr, *devfreQ = nullptr;
    ExpectLocalIn(gpu, &devdatP, &devctfP, &devdefO, &devsigP, npxl, slots, 0);
    ManagedArrayTexture mgr;
    ExpectLocalV3D(gpu, &mgr, vol.data(), vdim);
    std::vector<RFLOAT> outC(nP), outR((size_t)nP * nR), outT((size_t)nP * nT);
    for (int l = 0; l < nP; l++) {
        const int slot = l % slots;
        ExpectLocalP(gpu, devdatP, devctfP, devdefO, devsigP, dat.data(), ctf.data(), nullptr,
                     sig.data(), slot, l, npxl, 0);
        RFLOAT *wC, *wR, *wT, *wD;
        double *oldR, *oldT, *oldD, *trans, *rotq, *dpara;
        ExpectLocalHostA(gpu, &wC, &wR, &wT, &wD, &oldR, &oldT, &oldD, &trans, &rotq, &dpara, nR,
                         nT, 1, 0);
        ManagedCalPoint mcp;
        mcp.Init(1, 0, gpu, nR, nT, 1, npxl);
        std::memcpy(rotq, &rot[(size_t)l * nR * 4], sizeof(double) * nR * 4);
        std::memcpy(trans, &trs[(size_t)l * nT * 2], sizeof(double) * nT * 2);
        std::memcpy(oldR, &oR[(size_t)l * nR], sizeof(double) * nR);
        std::memcpy(oldT, &oT[(size_t)l * nT], sizeof(double) * nT);
        oldD[0] = 1;
        dpara[0] = 1;
        ExpectLocalRTD(gpu, &mcp, oldR, oldT, oldD, trans, rotq, dpara);
        ExpectLocalPreI3D(gpu, slot, &mgr, &mcp, devdefO, devfreQ, deviCol, deviRow, 0, 0, 0, 0,
                          pf, box, vdim, npxl, 1);
        ExpectLocalM(gpu, slot, &mcp, devdatP, devctfP, devsigP, wC, wR, wT, wD, 1.0, npxl);
        outC[l] = wC[0];
        std::memcpy(&outR[(size_t)l * nR], wR, sizeof(RFLOAT) * nR);
        std::memcpy(&outT[(size_t)l * nT], wT, sizeof(RFLOAT) * nT);
        ExpectLocalHostF(gpu, &wC, &wR, &wT, &wD, &oldR, &oldT, &oldD, &trans, &rotq, &dpara, 0);
    }
    ExpectLocalFin(gpu, &devdatP, &devctfP, &devdefO, &devfreQ, &devsigP, 0);
    ExpectFreeIdx(gpu, &deviCol, &deviRow);
    save(dir, "out_wC.bin", outC.data(), outC.size());
    save(dir, "out_wR.bin", outR.data(), outR.size());
    save(dir, "out_wT.bin", outT.data(), outT.size());

    // ------------------------------------------- 2-D local expectation
    // (ExpectLocalV2D, then per image the same sequence with PreI2D and a
    // ManagedCalPoint of mode 0, the rotations as (cos, sin) pairs)
    {
        const size_t n2 = (size_t)vdim * (vdim / 2 + 1);
        auto img2 = load<Complex>(dir, "vol2d.bin", n2);
        auto rot2 = load<double>(dir, "rot2d.bin", (size_t)nP * nR * 2);
        ExpectPreidx(gpu, &deviCol, &deviRow, iCol.data(), iRow.data(), npxl);
        ExpectLocalIn(gpu, &devdatP, &devctfP, &devdefO, &devsigP, npxl, slots, 0);
        ManagedArrayTexture mgr2;
        ExpectLocalV2D(gpu, &mgr2, img2.data(), (int)n2);
        for (int l = 0; l < nP; l++) {
            const int slot = l % slots;
            ExpectLocalP(gpu, devdatP, devctfP, devdefO, devsigP, dat.data(), ctf.data(),
                         nullptr, sig.data(), slot, l, npxl, 0);
            RFLOAT *wC, *wR, *wT, *wD;
            double *oldR, *oldT, *oldD, *trans, *rotq, *dpara;
            ExpectLocalHostA(gpu, &wC, &wR, &wT, &wD, &oldR, &oldT, &oldD, &trans, &rotq, &dpara,
                             nR, nT, 1, 0);
            ManagedCalPoint mcp;
            mcp.Init(0, 0, gpu, nR, nT, 1, npxl);
            std::memcpy(rotq, &rot2[(size_t)l * nR * 2], sizeof(double) * nR * 2);
            std::memcpy(trans, &trs[(size_t)l * nT * 2], sizeof(double) * nT * 2);
            std::memcpy(oldR, &oR[(size_t)l * nR], sizeof(double) * nR);
            std::memcpy(oldT, &oT[(size_t)l * nT], sizeof(double) * nT);
            oldD[0] = 1;
            dpara[0] = 1;
            ExpectLocalRTD(gpu, &mcp, oldR, oldT, oldD, trans, rotq, dpara);
            ExpectLocalPreI2D(gpu, slot, &mgr2, &mcp, devdefO, devfreQ, deviCol, deviRow, 0, 0, 0,
                              0, pf, box, vdim, npxl, 1);
            ExpectLocalM(gpu, slot, &mcp, devdatP, devctfP, devsigP, wC, wR, wT, wD, 1.0, npxl);
            outC[l] = wC[0];
            std::memcpy(&outR[(size_t)l * nR], wR, sizeof(RFLOAT) * nR);
            std::memcpy(&outT[(size_t)l * nT], wT, sizeof(RFLOAT) * nT);
            ExpectLocalHostF(gpu, &wC, &wR, &wT, &wD, &oldR, &oldT, &oldD, &trans, &rotq, &dpara,
                             0);
        }
        ExpectLocalFin(gpu, &devdatP, &devctfP, &devdefO, &devfreQ, &devsigP, 0);
        ExpectFreeIdx(gpu, &deviCol, &deviRow);
        save(dir, "out2_wC.bin", outC.data(), outC.size());
        save(dir, "out2_wR.bin", outR.data(), outR.size());
        save(dir, "out2_wT.bin", outT.data(), outT.size());
    }

    // ------------------------------------------------------------ insertion
    auto nr = load<double>(dir, "ins_rot.bin", (size_t)nP * mReco * 4);
    auto nt = load<double>(dir, "ins_trans.bin", (size_t)nP * mReco * 2);
    auto offS = load<double>(dir, "offs.bin", (size_t)nP * 2);
    auto w = load<RFLOAT>(dir, "w.bin", nP);
    auto nc = load<int>(dir, "nc.bin", nP);
    std::vector<int> iColPad(npxl), iRowPad(npxl);
    for (int p = 0; p < npxl; p++) {
        iColPad[p] = iCol[p] * pf;
        iRowPad[p] = iRow[p] * pf;
    }
    MPI_Comm hemi = 0, slav = 0;
    for (int form = 1; form <= 2; form++) {
        Volume F(vdim), T(vdim);
        double O3D[3] = {0, 0, 0};
        int counter = 0;
        g_reduced = 0;
        if (form == 1)
            InsertFT(F, T, O3D, &counter, hemi, slav, dat.data(), ctf.data(), sig.data(), nullptr,
                     offS.data(), w.data(), nr.data(), nt.data(), nullptr, iColPad.data(),
                     iRowPad.data(), 1.0f, false, pf, npxl, mReco, box, (int)F.sizeFT(), nP);
        else
            InsertFT(F, T, O3D, &counter, hemi, slav, dat.data(), ctf.data(), sig.data(), nullptr,
                     offS.data(), w.data(), nr.data(), nt.data(), nullptr, nc.data(),
                     iColPad.data(), iRowPad.data(), 1.0f, false, pf, npxl, mReco, box,
                     (int)F.sizeFT(), nP);
        std::vector<RFLOAT> Tr(nvox);
        for (size_t i = 0; i < nvox; i++) Tr[i] = REAL(T[i]);
        const std::string tag = std::to_string(form);
        save(dir, ("out_F" + tag + ".bin").c_str(), &F[0], nvox);
        save(dir, ("out_T" + tag + ".bin").c_str(), Tr.data(), nvox);
        save(dir, ("out_O" + tag + ".bin").c_str(), O3D, 3);
        save(dir, ("out_c" + tag + ".bin").c_str(), &counter, 1);
        save(dir, ("out_red" + tag + ".bin").c_str(), &g_reduced, 1);
    }
    std::printf("driver ok\n");
    return 0;
}
