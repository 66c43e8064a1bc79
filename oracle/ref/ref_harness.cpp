/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE.  extern "C" entry points over the
 * reference's own compiled sources (Makefile in this folder), used only to
 * pin the oracle restatement (oracle/tg3_oracle.c) and to make the golden
 * fixtures in tests/golden/.  Each entry point calls the reference routine
 * named in its comment; the loops around them follow the reference caller
 * cited beside them.  All arithmetic is the reference's, in double precision.
 */
#include <cstdlib>
#include <cstring>
#include <vector>

#include <boost/bind.hpp>

#include "ImageFile.h"
#include "Logging.h"
#include "Mask.h"
#include "Spectrum.h"
#include "Precision.h"
#include "Functions.h"
#include "TabFunction.h"
#include "CTF.h"
#include "Euler.h"
#include "ImageFunctions.h"
#include "Volume.h"
#include "Projector.h"
#include "Particle.h"
#include "Transformation.h"

/* The reconstruction entry loads the accumulators the reference keeps as
 * private members (_F3D, _T3D); the class is opened for this file only. */
#define private public
#define protected public
#include "Reconstructor.h"
#undef private
#undef protected

INITIALIZE_EASYLOGGINGPP

/* The loggers the reconstruction writes to, registered and silenced. */
static struct RefLoggers {
    RefLoggers()
    {
        static el::Configurations conf;
        conf.setToDefault();
        conf.set(el::Level::All, el::ConfigurationType::Enabled, "false");
        conf.set(el::Level::All, el::ConfigurationType::ToFile, "false");
        conf.set(el::Level::All, el::ConfigurationType::ToStandardOutput, "false");
        el::Loggers::setDefaultConfigurations(conf, true);
        const char* names[] = {"LOGGER_SYS", "LOGGER_RECO", "LOGGER_MPI", "LOGGER_FFT"};
        for (const char* n : names) el::Loggers::getLogger(n);
    }
} g_ref_loggers;

/* Defined in src/Optimiser.cpp (non-static, no header declaration). */
RFLOAT logDataVSPrior_m_huabin(const Complex* dat, const Complex* pri,
                               const RFLOAT* ctf, const RFLOAT* sigRcp,
                               const int m);
RFLOAT* logDataVSPrior_m_n_huabin(const Complex* dat, const Complex* pri,
                                  const RFLOAT* ctf, const RFLOAT* sigRcp,
                                  const int n, const int m, RFLOAT* result);

/* ---- stand-ins for the external calls the compared routines make -------- */

/* Particle::resample / Particle::shuffle draw their randomness through these
 * two GSL calls; the harness injects the permutation and u0 instead. */
static std::vector<size_t> g_perm;
static double g_u0 = 0;
static double g_flat_b = -1;

static char g_engine_dummy[64];
gsl_rng* get_random_engine() { return (gsl_rng*)g_engine_dummy; }

extern "C" void gsl_ran_shuffle(const gsl_rng*, void* base, size_t n, size_t size)
{
    if (size != sizeof(size_t) || n != g_perm.size()) abort();
    memcpy(base, g_perm.data(), n * sizeof(size_t));
}

extern "C" double gsl_ran_flat(const gsl_rng*, const double a, const double b)
{
    g_flat_b = b;
    return a + g_u0;
}

/* ---- entry points ------------------------------------------------------- */

extern "C" {

/* rotate3D(dmat33&, const dvec4&), src/Geometry/Euler.cpp:181-189 */
void ref_rotmat(const double* quat, int n, double* mat)
{
    for (int r = 0; r < n; r++) {
        dmat33 R;
        dvec4 q(quat[4 * r], quat[4 * r + 1], quat[4 * r + 2], quat[4 * r + 3]);
        rotate3D(R, q);
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) mat[9 * r + 3 * i + j] = R(i, j);
    }
}

/* Projector::project(Complex*, const dmat33&, iCol, iRow, nPxl, nThread),
 * src/Projector.cpp:356-374, on a projectee volume set directly in Fourier
 * space (vdim^3 padded grid, half-FT storage). */
void ref_project(const double* vol, int vdim, const double* mat, int nR,
                 const int* iCol, const int* iRow, int K, int pf, double* out)
{
    Projector proj;
    proj.setMode(MODE_3D);
    proj.setPf(pf);
    proj.setInterp(LINEAR_INTERP);
    Volume v(vdim, vdim, vdim, FT_SPACE);
    memcpy(&v[0], vol, sizeof(Complex) * v.sizeFT());
    const_cast<Volume&>(proj.projectee3D()).swap(v);
    for (int r = 0; r < nR; r++) {
        dmat33 R;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) R(i, j) = mat[9 * r + 3 * i + j];
        proj.project((Complex*)(out + 2 * (size_t)r * K), R, iCol, iRow, K, 1);
    }
}

/* Image::getByInterpolationFT(iCol, iRow, LINEAR_INTERP),
 * src/Image/Image.cpp:345-368, on a 2-D half transform set directly in
 * Fourier space, at the in-plane rotation (c, s) of the reference's 2-D
 * projector (gpu/src/Kernel.cu:786-819). */
void ref_project2d(const double* img, int vdim, const double* rot, int nR, const int* iCol,
                   const int* iRow, int K, int pf, double* out)
{
    Image I(vdim, vdim, FT_SPACE);
    memcpy(&I[0], img, sizeof(Complex) * I.sizeFT());
    for (int r = 0; r < nR; r++) {
        const double c = rot[2 * r], s = rot[2 * r + 1];
        for (int p = 0; p < K; p++) {
            const double i = (double)(iCol[p] * pf), j = (double)(iRow[p] * pf);
            const Complex v = I.getByInterpolationFT(i * c - j * s, i * s + j * c, LINEAR_INTERP);
            out[2 * ((size_t)r * K + p)] = REAL(v);
            out[2 * ((size_t)r * K + p) + 1] = IMAG(v);
        }
    }
}

/* One 2-D insertion through Image::addFT(Complex / RFLOAT, iCol, iRow),
 * src/Image/Image.cpp:370-402: img times ctf times w into F, ctf^2 w into T,
 * at the in-plane rotation (c, s) of the padded pixel (iColPad, iRowPad). */
void ref_insert2d(double* F, double* T, int vdim, const double* img, const double* ctf, double c,
                  double s, double w, const int* iColPad, const int* iRowPad, int K)
{
    Image IF(vdim, vdim, FT_SPACE), IT(vdim, vdim, FT_SPACE);
    memcpy(&IF[0], F, sizeof(Complex) * IF.sizeFT());
    for (size_t i = 0; i < IT.sizeFT(); i++) IT[i] = COMPLEX(T[i], 0);
    for (int p = 0; p < K; p++) {
        const double a = iColPad[p], b = iRowPad[p];
        const double x = c * a - s * b, y = s * a + c * b;
        const Complex v = COMPLEX(img[2 * p] * ctf[p] * w, img[2 * p + 1] * ctf[p] * w);
        IF.addFT(v, x, y);
        IT.addFT(ctf[p] * ctf[p] * w, x, y);
    }
    memcpy(F, &IF[0], sizeof(Complex) * IF.sizeFT());
    for (size_t i = 0; i < IT.sizeFT(); i++) T[i] = REAL(IT[i]);
}

/* ImageFile::readMetaData + readImage(dst, iSlc), src/Image/ImageFile.cpp:
 * 209-290: section iSlc of an MRC stack in the reference's in-memory layout
 * (the file's centre pixel at index 0).  Returns non-zero on a size mismatch. */
int ref_read_mrc(const char* path, int iSlc, int N, double* out)
{
    ImageFile imf(path, "rb");
    imf.readMetaData();
    Image img;
    imf.readImage(img, iSlc);
    if (img.nColRL() != N || img.nRowRL() != N) return 1;
    for (size_t i = 0; i < img.sizeRL(); i++) out[i] = img.iGetRL(i);
    return 0;
}

/* One image through Optimiser::substractBgImg (bgMeanStddev), statImg's
 * bgStddev about 0 and maskImg with zeroMask (softMask to 0, edge
 * EDGE_WIDTH_RL), src/Optimiser.cpp:4796-4985; in / out in the in-memory
 * layout; stats = (background mean, deviation, normalised deviation). */
void ref_prep_image(const double* in, int N, double r, int mask, double* out, double* stats)
{
    Image img(N, N, RL_SPACE);
    for (size_t i = 0; i < img.sizeRL(); i++) img(i) = in[i];
    RFLOAT m, s;
    bgMeanStddev(m, s, img, r);
    for (size_t i = 0; i < img.sizeRL(); i++) {
        img(i) -= m;
        img(i) /= s;
    }
    stats[0] = m;
    stats[1] = s;
    stats[2] = bgStddev(0, img, r);
    if (mask) softMask(img, img, (RFLOAT)r, (RFLOAT)EDGE_WIDTH_RL, (RFLOAT)0, 1u);
    for (size_t i = 0; i < img.sizeRL(); i++) out[i] = img(i);
}

/* FFT::fw(Image&, nThread), src/FFT.cpp:118-140, through the vendored FFTW:
 * the unnormalised r2c transform of an N x N image given in the Image's own
 * storage order (its centre at index 0, as Optimiser::fwImg transforms it,
 * src/Optimiser.cpp:5003-5013); out: the half transform [N][N/2 + 1]. */
void ref_fw_image(const double* in, int N, double* out)
{
    Image img(N, N, RL_SPACE);
    for (size_t i = 0; i < img.sizeRL(); i++) img(i) = in[i];
    FFT fft;
    fft.fw(img, 1);
    for (size_t i = 0; i < img.sizeFT(); i++) {
        out[2 * i] = img[i].dat[0];
        out[2 * i + 1] = img[i].dat[1];
    }
}

/* Optimiser::reMaskImg, src/Optimiser.cpp:6053-6111: the mask
 * softMask(mask, r, ew) (src/Functions/Mask.cpp:333-350), then for the
 * image FFT::bw (normalised), MUL_RL by the mask and FFT::fw.  ft: the half
 * transform [N][N/2 + 1] complex, in place. */
void ref_remask(double* ft, int N, double r, double ew)
{
    Image img(N, N, FT_SPACE);
    for (size_t i = 0; i < img.sizeFT(); i++) {
        img[i].dat[0] = ft[2 * i];
        img[i].dat[1] = ft[2 * i + 1];
    }
    Image mask(N, N, RL_SPACE);
    softMask(mask, (RFLOAT)r, (RFLOAT)ew, 1u);
    FFT fft;
    fft.bw(img, 1);
    MUL_RL(img, mask);
    fft.fw(img, 1);
    for (size_t i = 0; i < img.sizeFT(); i++) {
        ft[2 * i] = img[i].dat[0];
        ft[2 * i + 1] = img[i].dat[1];
    }
}

/* powerSpectrum(vec&, const Image&, r, nThread), src/Functions/Spectrum.cpp:
 * 161-190, of a half transform ft [N][N/2 + 1] complex; out [r]. */
void ref_power_spectrum(const double* ft, int N, int r, double* out)
{
    Image img(N, N, FT_SPACE);
    memcpy(&img[0], ft, sizeof(Complex) * img.sizeFT());
    vec ps(r);
    powerSpectrum(ps, img, r, 1);
    for (int i = 0; i < r; i++) out[i] = ps(i);
}

/* translate(Complex*, nTransCol, nTransRow, nCol, nRow, iCol, iRow, nPxl,
 * nThread), src/Image/ImageFunctions.cpp:233-252 */
void ref_translate(const double* trans, int nT, int N, const int* iCol,
                   const int* iRow, int K, double* out)
{
    for (int t = 0; t < nT; t++)
        translate((Complex*)(out + 2 * (size_t)t * K), trans[2 * t],
                  trans[2 * t + 1], N, N, iCol, iRow, K, 1);
}

/* translate(Complex* dst, const Complex* src, ...),
 * src/Image/ImageFunctions.cpp:471-492 */
void ref_translate_image(const double* src, double tx, double ty, int N,
                         const int* iCol, const int* iRow, int K, double* dst)
{
    translate((Complex*)dst, (const Complex*)src, tx, ty, N, N, iCol, iRow, K, 1);
}

/* CTF(RFLOAT*, ...), src/CTF.cpp:98-145; attr in CTFAttr field order */
void ref_ctf(const double* attr, double pixelSize, int N, const int* iCol,
             const int* iRow, int K, double* out)
{
    CTF(out, pixelSize, attr[0], attr[1], attr[2], attr[3], attr[4], attr[5],
        attr[6], N, N, iCol, iRow, K);
}

/* logDataVSPrior_m_huabin, src/Optimiser.cpp:8922-8946 */
double ref_logdvp(const double* dat, const double* pri, const double* ctf,
                  const double* sigRcp, int K)
{
    return logDataVSPrior_m_huabin((const Complex*)dat, (const Complex*)pri,
                                   ctf, sigRcp, K);
}

/* logDataVSPrior_m_n_huabin (pixel-major, n images),
 * src/Optimiser.cpp:9666-9707 */
void ref_logdvp_mn(const double* dat, const double* pri, const double* ctf,
                   const double* sigRcp, int nImg, int K, double* result)
{
    memset(result, 0, sizeof(double) * nImg);
    logDataVSPrior_m_n_huabin((const Complex*)dat, (const Complex*)pri, ctf,
                              sigRcp, nImg, K, result);
}

/* TabFunction::init(MKB_FT_R2(., a, alpha), 0, b, n), src/TabFunction.cpp:25-39
 * with MKB_FT_R2, src/Functions/Functions.cpp:108-126; read back through
 * TabFunction::operator() at the grid points. */
void ref_mkb_table(double a, double alpha, double b, int n, double* tab)
{
    TabFunction tf;
    tf.init(boost::bind(MKB_FT_R2, boost::placeholders::_1, a, alpha), 0, b, n);
    double s = b / n;
    for (int i = 0; i <= n; i++) tab[i] = tf(i * s);
}

/* Reconstructor::insertP's per-pixel loop, src/Reconstructor.cpp:807-862,
 * calling the reference's Volume::addFT:
 *   kernel 1: addFT(value, x, y, z, a, TabFunction), src/Image/Volume.cpp:399-431
 *   kernel 0: addFT(value, x, y, z) (trilinear), src/Image/Volume.cpp:334-369
 * F is complex [vdim][vdim][vdim/2+1]; T real of the same shape (stored in the
 * real part of a complex Volume in the reference). */
void ref_insert(double* F, double* T, int vdim, const double* img,
                const double* ctf, const double* mat, double w,
                const int* iColPad, const int* iRowPad, int K, int kernel,
                double a, double alpha, double tabB, int tabN)
{
    Volume vF(vdim, vdim, vdim, FT_SPACE), vT(vdim, vdim, vdim, FT_SPACE);
    const size_t n = vF.sizeFT();
    for (size_t i = 0; i < n; i++) {
        vF[i].dat[0] = F[2 * i];
        vF[i].dat[1] = F[2 * i + 1];
        vT[i].dat[0] = T[i];
        vT[i].dat[1] = 0;
    }
    TabFunction tf;
    tf.init(boost::bind(MKB_FT_R2, boost::placeholders::_1, a, alpha), 0, tabB, tabN);
    const double pfa = sqrt(tabB);
    for (int i = 0; i < K; i++) {
        double oldCor[3];
        double c = iColPad[i], r = iRowPad[i];
        /* rotation as applied by insertP: oldCor = R (iCol, iRow, 0) */
        oldCor[0] = mat[0] * c + mat[1] * r;
        oldCor[1] = mat[3] * c + mat[4] * r;
        oldCor[2] = mat[6] * c + mat[7] * r;
        Complex src;
        src.dat[0] = img[2 * i];
        src.dat[1] = img[2 * i + 1];
        Complex val = src * ctf[i] * w;
        double tval = ctf[i] * ctf[i] * w;
        if (kernel == 1) {
            vF.addFT(val, oldCor[0], oldCor[1], oldCor[2], pfa, tf);
            vT.addFT(tval, oldCor[0], oldCor[1], oldCor[2], pfa, tf);
        } else {
            vF.addFT(val, oldCor[0], oldCor[1], oldCor[2]);
            vT.addFT(tval, oldCor[0], oldCor[1], oldCor[2]);
        }
    }
    for (size_t i = 0; i < n; i++) {
        F[2 * i] = vF[i].dat[0];
        F[2 * i + 1] = vF[i].dat[1];
        T[i] = vT[i].dat[0];
    }
}

/* Particle rotation-axis narrowing + resampling, as Optimiser::updateSP runs
 * them (src/Optimiser.cpp:1357-1396): setUR, [setPeakFactor(PAR_R),]
 * keepHalfHeightPeak(PAR_R), resample(nOut, PAR_R)
 * (src/Particle.cpp:1864-1973, 1275-1463).  The shuffle permutation and u0
 * are injected.  Row i of the particle's quaternion matrix carries i in its
 * first component so that the source of every resampled row can be read
 * back.  mode: 0 = no narrowing, 1 = setPeakFactor + keepHalfHeightPeak.
 * Returns the b bound that resample passed to gsl_ran_flat. */
double ref_resample(int n, const double* u, const double* w, const size_t* perm,
                    double u0, int nOut, int mode, int* src, double* wOut)
{
    Particle par;
    par.setMode(MODE_3D);
    par.setNR(n);
    dmat4 r = dmat4::Zero(n, 4);
    dvec wR(n), uR(n);
    for (int i = 0; i < n; i++) {
        r(i, 0) = i;
        wR(i) = w[i];
        uR(i) = u[i];
    }
    par.setR(r);
    par.setWR(wR);
    par.setUR(uR);
    if (mode == 1) {
        par.setPeakFactor(PAR_R);
        par.keepHalfHeightPeak(PAR_R);
    }
    g_perm.assign(perm, perm + n);
    g_u0 = u0;
    par.resample(nOut, PAR_R);
    dmat4 ro = par.r();
    dvec wo = par.wR();
    for (int j = 0; j < nOut; j++) {
        src[j] = (int)ro(j, 0);
        wOut[j] = wo(j);
    }
    return g_flat_b;
}

/* d_index_sort_descend (gsl_sort_largest_index),
 * src/Functions/Functions.cpp:72-79 */
/* SYMMETRIZE_FT (include/Geometry/Transformation.h:170-196) with the
 * elements given as matrices: the volume plus, for every R,
 * VOL_TRANSFORM_MAT_FT(se, src, R, r, LINEAR_INTERP) of the original.  vol
 * complex [vdim][vdim][vdim/2 + 1], in place; mats [nSym][9] row-major. */
void ref_symmetrize(double* vol, int vdim, const double* mats, int nSym, double r)
{
    Volume src(vdim, vdim, vdim, FT_SPACE);
    const size_t n = src.sizeFT();
    for (size_t i = 0; i < n; i++) {
        src[i].dat[0] = vol[2 * i];
        src[i].dat[1] = vol[2 * i + 1];
    }
    Volume result = src.copyVolume();
    Volume se(vdim, vdim, vdim, FT_SPACE);
    for (int s = 0; s < nSym; s++) {
        dmat33 R;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) R(a, b) = mats[9 * s + 3 * a + b];
        VOL_TRANSFORM_MAT_FT(se, src, R, r, LINEAR_INTERP, 1);
        ADD_FT(result, se);
    }
    for (size_t i = 0; i < n; i++) {
        vol[2 * i] = result[i].dat[0];
        vol[2 * i + 1] = result[i].dat[1];
    }
}

/* Reconstructor::reconstruct(Volume&, nThread), src/Reconstructor.cpp:1129-1790,
 * on accumulators set directly: F complex and T real on the padded half grid
 * ([vdim][vdim][vdim/2 + 1] in 3-D, [vdim][vdim/2 + 1] in 2-D, vdim = N pf),
 * with the MAP Wiener step from fsc (nFsc shells), W balancing against the
 * MKB kernel (gridCorr != 0) or W = 1/T, and the real-space correction the
 * build configures (include/Config.h: trilinear).  The reconstructing rank
 * is a non-master rank (the master returns at once).  out: the N^d map,
 * coordinate i at index i + N/2, slowest axis first.  Returns 0. */
int ref_reconstruct(int dim, int N, int pf, double a, double alpha, int maxRadius,
                    const double* F, const double* T, const double* fsc, int nFsc,
                    int joinHalf, int gridCorr, int nThread, double* out)
{
    Reconstructor R;
    R.setCommRank(1);
    R.setCommSize(2);
    R.init(dim == 2 ? MODE_2D : MODE_3D, N, N, pf, NULL, a, alpha);
    R.allocSpace(nThread);
    R.setMaxRadius(maxRadius);
    R.setMAP(true);
    R.setGridCorr(gridCorr != 0);
    R.setJoinHalf(joinHalf != 0);
    vec v(nFsc);
    for (int i = 0; i < nFsc; i++) v(i) = fsc[i];
    R.setFSC(v);
    const int vdim = N * pf;
    Complex* pF = dim == 2 ? &R._F2D[0] : &R._F3D[0];
    Complex* pT = dim == 2 ? &R._T2D[0] : &R._T3D[0];
    const size_t n = dim == 2 ? R._F2D.sizeFT() : R._F3D.sizeFT();
    if (n != (size_t)(dim == 2 ? 1 : vdim) * vdim * (vdim / 2 + 1)) return 1;
    for (size_t i = 0; i < n; i++) {
        pF[i].dat[0] = F[2 * i];
        pF[i].dat[1] = F[2 * i + 1];
        pT[i].dat[0] = T[i];
        pT[i].dat[1] = 0;
    }
    Volume dst;
    R.reconstruct(dst, nThread);
    const int h = N / 2;
    if (dim == 2) {
        for (int j = -h; j < N - h; j++)
            for (int i = -h; i < N - h; i++)
                out[(size_t)(j + h) * N + (i + h)] = dst.getRL(i, j, 0);
    } else {
        for (int k = -h; k < N - h; k++)
            for (int j = -h; j < N - h; j++)
                for (int i = -h; i < N - h; i++)
                    out[((size_t)(k + h) * N + (j + h)) * N + (i + h)] = dst.getRL(i, j, k);
    }
    return 0;
}

void ref_sort_descend(const double* v, int n, size_t* idx)
{
    dvec d(n);
    for (int i = 0; i < n; i++) d(i) = v[i];
    uvec o = d_index_sort_descend(d);
    for (int i = 0; i < n; i++) idx[i] = o(i);
}

} /* extern "C" */
