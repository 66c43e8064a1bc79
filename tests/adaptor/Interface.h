/*
 * Stand-in for THUNDER's gpu/interface/Interface.h and the types its
 * signatures use, so that the drop-in adaptor (interface/Interface.cpp) can
 * be compiled and run where the reference tree is absent.  TEST
 * INFRASTRUCTURE: only tests/test_gpu_adaptor.py builds it.
 *
 * The layouts are the reference's single-precision ones: Complex is two
 * RFLOATs (include/Precision.h:77-99), CTFAttr seven RFLOATs
 * (include/Database.h:108-122), a Volume holds the half transform
 * [nSlc][nSlc][nSlc / 2 + 1] of Complex (include/Image/Volume.h) and an
 * Image the half transform [n][n / 2 + 1] (include/Image/Image.h); the
 * handles carry only what the adaptor reads (ManagedCalPoint's hypothesis
 * counts, gpu/include/ManagedCalPoint.h:15-51).  The function declarations
 * repeat the reference's signatures, which the adaptor defines.
 */
#ifndef TG3_TEST_INTERFACE_H
#define TG3_TEST_INTERFACE_H

#include <cstddef>
#include <vector>

#include "mpi.h"

typedef float RFLOAT;

struct Complex {
    RFLOAT dat[2];
};
inline RFLOAT REAL(const Complex& c) { return c.dat[0]; }
inline Complex COMPLEX(RFLOAT a, RFLOAT b) { return Complex{{a, b}}; }

struct CTFAttr {
    RFLOAT voltage, defocusU, defocusV, defocusTheta, Cs, amplitudeContrast, phaseShift;
};

class Volume {
public:
    explicit Volume(int n) : n_(n), d_((size_t)n * n * (n / 2 + 1), Complex{{0, 0}}) {}
    size_t sizeFT() const { return d_.size(); }
    int nSlcFT() const { return n_; }
    Complex& operator[](size_t i) { return d_[i]; }

private:
    int n_;
    std::vector<Complex> d_;
};

class Image {
public:
    explicit Image(int n) : d_((size_t)n * (n / 2 + 1), Complex{{0, 0}}) {}
    Complex& operator[](size_t i) { return d_[i]; }

private:
    std::vector<Complex> d_;
};

class ManagedArrayTexture {};

class ManagedCalPoint {
public:
    void Init(int mode, int cSearch, int gpuIdx, int nR, int nT, int mD, int npxl)
    {
        mode_ = mode;
        (void)cSearch;
        (void)gpuIdx;
        (void)npxl;
        nR_ = nR;
        nT_ = nT;
        mD_ = mD;
    }
    int getNR() { return nR_; }
    int getNT() { return nT_; }
    int getMD() { return mD_; }
    int getMode() { return mode_; }

private:
    int nR_ = 0, nT_ = 0, mD_ = 0, mode_ = 1;
};

void getAviDevice(std::vector<int>& gpus);
void ExpectPreidx(int gpuIdx, int** deviCol, int** deviRow, int* iCol, int* iRow, int npxl);
void ExpectPrefre(int gpuIdx, RFLOAT** devfreQ, RFLOAT* freQ, int npxl);
void ExpectLocalIn(int gpuIdx, Complex** devdatP, RFLOAT** devctfP, RFLOAT** devdefO,
                   RFLOAT** devsigP, int nPxl, int cpyNumL, int searchType);
void ExpectLocalV2D(int gpuIdx, ManagedArrayTexture* mgr, Complex* volume, int dimSize);
void ExpectLocalV3D(int gpuIdx, ManagedArrayTexture* mgr, Complex* volume, int vdim);
void ExpectLocalP(int gpuIdx, Complex* devdatP, RFLOAT* devctfP, RFLOAT* devdefO,
                  RFLOAT* devsigP, Complex* datP, RFLOAT* ctfP, RFLOAT* defO, RFLOAT* sigP,
                  int threadId, int imgId, int npxl, int cSearch);
void ExpectLocalHostA(int gpuIdx, RFLOAT** wC, RFLOAT** wR, RFLOAT** wT, RFLOAT** wD,
                      double** oldR, double** oldT, double** oldD, double** trans,
                      double** rot, double** dpara, int mR, int mT, int mD, int cSearch);
void ExpectLocalRTD(int gpuIdx, ManagedCalPoint* mcp, double* oldR, double* oldT, double* oldD,
                    double* trans, double* rot, double* dpara);
void ExpectLocalPreI2D(int gpuIdx, int datShift, ManagedArrayTexture* mgr, ManagedCalPoint* mcp,
                       RFLOAT* devdefO, RFLOAT* devfreQ, int* deviCol, int* deviRow,
                       RFLOAT phaseShift, RFLOAT conT, RFLOAT k1, RFLOAT k2, int pf, int idim,
                       int vdim, int npxl, int interp);
void ExpectLocalPreI3D(int gpuIdx, int datShift, ManagedArrayTexture* mgr, ManagedCalPoint* mcp,
                       RFLOAT* devdefO, RFLOAT* devfreQ, int* deviCol, int* deviRow,
                       RFLOAT phaseShift, RFLOAT conT, RFLOAT k1, RFLOAT k2, int pf, int idim,
                       int vdim, int npxl, int interp);
void ExpectLocalM(int gpuIdx, int datShift, ManagedCalPoint* mcp, Complex* devdatP,
                  RFLOAT* devctfP, RFLOAT* devsigP, RFLOAT* wC, RFLOAT* wR, RFLOAT* wT,
                  RFLOAT* wD, double oldC, int npxl);
void ExpectLocalHostF(int gpuIdx, RFLOAT** wC, RFLOAT** wR, RFLOAT** wT, RFLOAT** wD,
                      double** oldR, double** oldT, double** oldD, double** trans,
                      double** rot, double** dpara, int cSearch);
void ExpectLocalFin(int gpuIdx, Complex** devdatP, RFLOAT** devctfP, RFLOAT** devdefO,
                    RFLOAT** devfreQ, RFLOAT** devsigP, int cSearch);
void ExpectFreeIdx(int gpuIdx, int** deviCol, int** deviRow);
void ReMask(std::vector<Image>& img, RFLOAT maskRadius, RFLOAT pixelSize, RFLOAT ew, int idim,
            int imgNum);
void PrepareTF(int gpuIdx, Volume& F3D, Volume& T3D, double* symMat, int nSymmetryElement,
               int maxRadius, int pf);
void InsertFT(Volume& F3D, Volume& T3D, double* O3D, int* counter, MPI_Comm& hemi,
              MPI_Comm& slav, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
              CTFAttr* ctfaData, double* offS, RFLOAT* w, double* nR, double* nT, double* nD,
              int* nC, const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch,
              int opf, int npxl, int mReco, int idim, int dimSize, int imgNum);
void InsertFT(Volume& F3D, Volume& T3D, double* O3D, int* counter, MPI_Comm& hemi,
              MPI_Comm& slav, Complex* datP, RFLOAT* ctfP, RFLOAT* sigRcpP,
              CTFAttr* ctfaData, double* offS, RFLOAT* w, double* nR, double* nT, double* nD,
              const int* iCol, const int* iRow, RFLOAT pixelSize, bool cSearch, int opf,
              int npxl, int mReco, int idim, int dimSize, int imgNum);

#endif
