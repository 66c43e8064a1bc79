/*
 * tg3_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A double-precision CPU restatement of the THUNDER E-step and insertion hot
 * path.  Only tests/, __graft_entry__.smoke() and bench.py (its CPU-baseline
 * leg and its `--impl reference` arm) may load this library, and only as the
 * checker or the timed CPU baseline.  The shipped library never links it.
 *
 * Every function cites the reference routine it restates (paths are relative
 * to the THUNDER source tree).  The restatement is pinned against the
 * reference's own sources compiled by oracle/ref/Makefile (outputs compared in
 * tests/test_oracle_pin.py) and against the committed fixtures in
 * tests/golden/ that the compiled reference produced.
 *
 * Conventions shared with the CUDA library:
 *  - complex arrays are interleaved (re, im) pairs;
 *  - a padded half-FT volume of edge vdim is stored [z][y][x] with
 *    x in [0, vdim/2], y and z in [0, vdim) and negative frequencies wrapped
 *    (Volume::iFTHalf, include/Image/Volume.h:566-573);
 *  - rotation matrices are row-major 3x3.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define OR_EXPORT __attribute__((visibility("default")))

/* ---------------------------------------------------------------------------
 * Pixel selection.  Optimiser::allocPreCalIdx, src/Optimiser.cpp:7942-7992:
 * half-plane pixels (skip i == 0 && j < 0) with rL^2 <= i^2 + j^2 < rU^2 and
 * rL <= rint(|k|) < rU, visited j-outer / i-inner (IMAGE_FOR_PIXEL_R_FT,
 * include/Image/Image.h:68-70).  iPxl is Image::iFTHalf
 * (include/Image/Image.h:426-432).  Returns K, or -1 if maxn is too small.
 * ------------------------------------------------------------------------- */
OR_EXPORT int or_pixel_index(int size, double rU, double rL,
                             int* iCol, int* iRow, int* iSig, int* iPxl,
                             int maxn)
{
    const double r = rU + 1;
    const double rU2 = rU * rU, rL2 = rL * rL;
    const int nColFT = size / 2 + 1;
    int n = 0;
    for (int j = (int)(-r); j < r; j++)
        for (int i = 0; i <= r; i++) {
            if (i == 0 && j < 0) continue;
            double u = (double)i * i + (double)j * j;
            if (u < rU2 && u >= rL2) {
                int v = (int)rint(hypot((double)i, (double)j));
                if (v < rU && v >= rL) {
                    if (n >= maxn) return -1;
                    iCol[n] = i;
                    iRow[n] = j;
                    iSig[n] = v;
                    iPxl[n] = (j >= 0 ? j : j + size) * nColFT + i;
                    n++;
                }
            }
        }
    return n;
}

/* ---------------------------------------------------------------------------
 * Quaternion -> rotation matrix.  rotate3D(dmat33&, const dvec4&),
 * src/Geometry/Euler.cpp:181-189: R = I + 2 q0 A + 2 A A with
 * A = [[0,-q3,q2],[q3,0,-q1],[-q2,q1,0]].  Output row-major.
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_rotmat(const double* quat, int n, double* mat)
{
    for (int r = 0; r < n; r++) {
        const double* q = quat + 4 * r;
        double A[3][3] = {{0, -q[3], q[2]}, {q[3], 0, -q[1]}, {-q[2], q[1], 0}};
        double* m = mat + 9 * r;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                double aa = (2 * A[i][0]) * A[0][j] + (2 * A[i][1]) * A[1][j]
                          + (2 * A[i][2]) * A[2][j];
                m[3 * i + j] = ((i == j ? 1.0 : 0.0) + (2 * q[0]) * A[i][j]) + aa;
            }
    }
}

/* Index of voxel (x, y, z) of a half-FT volume with wrapped y, z
 * (Volume::iFTHalf, include/Image/Volume.h:566-573). */
static inline size_t vol_index(int vdim, int x, int y, int z)
{
    const size_t nx = (size_t)(vdim / 2 + 1);
    return ((size_t)(z >= 0 ? z : z + vdim) * (size_t)vdim
          + (size_t)(y >= 0 ? y : y + vdim)) * nx + (size_t)x;
}

/* ---------------------------------------------------------------------------
 * Trilinear Fourier-space sample with Friedel mirroring.
 * Volume::getByInterpolationFT, src/Image/Volume.cpp:308-332;
 * conjHalf(RFLOAT&...), include/Image/Volume.h:139-150;
 * WG_TRI_INTERP_LINEAR, include/Functions/Interpolation.h:155-199;
 * getFTHalf(w, x0), src/Image/Volume.cpp:481-553 (corner order k, j, i).
 * ------------------------------------------------------------------------- */
static void sample_trilinear(const double* vol, int vdim,
                             double x, double y, double z, double out[2])
{
    int conj = 0;
    if (x < 0) { x = -x; y = -y; z = -z; conj = 1; }
    double xs[3] = {x, y, z};
    int x0[3];
    double v[3][2];
    for (int d = 0; d < 3; d++) {
        x0[d] = (int)floor(xs[d]);
        double xd = xs[d] - x0[d];
        v[d][0] = 1 - xd;
        v[d][1] = xd;
    }
    double re = 0, im = 0;
    for (int k = 0; k < 2; k++)
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < 2; i++) {
                double w = v[0][i] * v[1][j] * v[2][k];
                size_t idx = vol_index(vdim, x0[0] + i, x0[1] + j, x0[2] + k);
                re += vol[2 * idx] * w;
                im += vol[2 * idx + 1] * w;
            }
    out[0] = re;
    out[1] = conj ? -im : im;
}

/* ---------------------------------------------------------------------------
 * Fourier-slice extraction.  Projector::project(Complex*, const dmat33&,
 * iCol, iRow, nPxl), src/Projector.cpp:356-374: P[p] =
 * trilinear(V, R (iCol*pf, iRow*pf, 0)).  out is [nR][K] complex.
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_project(const double* vol, int vdim, const double* mat,
                          int nR, const int* iCol, const int* iRow, int K,
                          int pf, double* out)
{
    for (int r = 0; r < nR; r++) {
        const double* m = mat + 9 * r;
        for (int p = 0; p < K; p++) {
            double a = (double)(iCol[p] * pf), b = (double)(iRow[p] * pf);
            double x = m[0] * a + m[1] * b + m[2] * 0.0;
            double y = m[3] * a + m[4] * b + m[5] * 0.0;
            double z = m[6] * a + m[7] * b + m[8] * 0.0;
            sample_trilinear(vol, vdim, x, y, z, out + 2 * ((size_t)r * K + p));
        }
    }
}

/* ---------------------------------------------------------------------------
 * 2-D: bilinear sample of a half transform [vdim][vdim/2 + 1] (rows in FFT
 * order) at (x, y), Image::getByInterpolationFT(iCol, iRow, LINEAR_INTERP),
 * src/Image/Image.cpp:345-368: x < 0 is read at (-x, -y) and conjugated
 * (conjHalf); WG_BI_INTERP_LINEAR weights; getFTHalf wraps negative rows.
 * ------------------------------------------------------------------------- */
static void sample_bilinear(const double* img, int vdim, double x, double y, double out[2])
{
    int conj = 0;
    if (x < 0) { x = -x; y = -y; conj = 1; }
    const int nx = vdim / 2 + 1;
    const int x0 = (int)floor(x), y0 = (int)floor(y);
    const double fx = x - x0, fy = y - y0;
    const double wx[2] = {1 - fx, fx}, wy[2] = {1 - fy, fy};
    double re = 0, im = 0;
    for (int j = 0; j < 2; j++)
        for (int i = 0; i < 2; i++) {
            int yy = y0 + j;
            if (yy < 0) yy += vdim;
            const size_t idx = (size_t)yy * nx + (x0 + i);
            re += img[2 * idx] * wx[i] * wy[j];
            im += img[2 * idx + 1] * wx[i] * wy[j];
        }
    out[0] = re;
    out[1] = conj ? -im : im;
}

/* 2-D projection: in-plane rotation (c, s) of the pixel (iCol pf, iRow pf),
 * the form of the reference's 2-D projector (kernel_Project2D,
 * gpu/src/Kernel.cu:786-819: x = i c - j s, y = i s + j c).  rot is
 * [nR][2] (c, s); out [nR][K] complex. */
OR_EXPORT void or_project2d(const double* img, int vdim, const double* rot, int nR,
                            const int* iCol, const int* iRow, int K, int pf, double* out)
{
    for (int r = 0; r < nR; r++) {
        const double c = rot[2 * r], s = rot[2 * r + 1];
        for (int p = 0; p < K; p++) {
            const double i = (double)(iCol[p] * pf), j = (double)(iRow[p] * pf);
            sample_bilinear(img, vdim, i * c - j * s, i * s + j * c,
                            out + 2 * ((size_t)r * K + p));
        }
    }
}

/* 2-D insertion of one slice: Image::addFT(value, iCol, iRow),
 * src/Image/Image.cpp:370-386 (bilinear, x < 0 at (-x, -y) conjugated) at the
 * in-plane rotation (c, s) of the padded pixel (iColPad, iRowPad):
 * F += w ctf img, T += w ctf^2, both [vdim][vdim/2 + 1]. */
OR_EXPORT void or_insert2d(double* F, double* T, int vdim, const double* img, const double* ctf,
                           double c, double s, double w, const int* iColPad,
                           const int* iRowPad, int K)
{
    const int nx = vdim / 2 + 1;
    for (int p = 0; p < K; p++) {
        const double a = iColPad[p], b = iRowPad[p];
        double x = c * a - s * b, y = s * a + c * b;
        double vr = img[2 * p] * ctf[p] * w, vi = img[2 * p + 1] * ctf[p] * w;
        const double vt = ctf[p] * ctf[p] * w;
        if (x < 0) { x = -x; y = -y; vi = -vi; }
        const int x0 = (int)floor(x), y0 = (int)floor(y);
        const double fx = x - x0, fy = y - y0;
        for (int j = 0; j < 2; j++)
            for (int i = 0; i < 2; i++) {
                const double ww = (i ? fx : 1 - fx) * (j ? fy : 1 - fy);
                int yy = y0 + j;
                if (yy < 0) yy += vdim;
                const size_t idx = (size_t)yy * nx + x0 + i;
                F[2 * idx] += vr * ww;
                F[2 * idx + 1] += vi * ww;
                T[idx] += vt * ww;
            }
    }
}

/* ---------------------------------------------------------------------------
 * Phase-shift bank.  translate(Complex*, nTransCol, nTransRow, nCol, nRow,
 * iCol, iRow, nPxl), src/Image/ImageFunctions.cpp:233-252:
 * S[p] = exp(-2 pi i (iCol tx / N + iRow ty / N)).  trans is [nT][2].
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_translate(const double* trans, int nT, int N,
                            const int* iCol, const int* iRow, int K,
                            double* out)
{
    for (int t = 0; t < nT; t++) {
        double rCol = trans[2 * t] / N, rRow = trans[2 * t + 1] / N;
        for (int p = 0; p < K; p++) {
            double phase = 2 * M_PI * (iCol[p] * rCol + iRow[p] * rRow);
            out[2 * ((size_t)t * K + p)] = cos(-phase);
            out[2 * ((size_t)t * K + p) + 1] = sin(-phase);
        }
    }
}

/* Shift an image by (tx, ty): dst = src * exp(-2 pi i k.t / N).
 * translate(Complex* dst, const Complex* src, ...),
 * src/Image/ImageFunctions.cpp:471-492. */
OR_EXPORT void or_translate_image(const double* src, double tx, double ty,
                                  int N, const int* iCol, const int* iRow,
                                  int K, double* dst)
{
    double rCol = tx / N, rRow = ty / N;
    for (int p = 0; p < K; p++) {
        double phase = 2 * M_PI * (iCol[p] * rCol + iRow[p] * rRow);
        double c = cos(-phase), s = sin(-phase);
        double a = src[2 * p], b = src[2 * p + 1];
        dst[2 * p] = a * c - b * s;
        dst[2 * p + 1] = a * s + b * c;
    }
}

/* ---------------------------------------------------------------------------
 * CTF at the selected pixels.  CTF(RFLOAT*, pixelSize, voltage, dU, dV,
 * theta, Cs, A, phaseShift, nCol, nRow, iCol, iRow, nPxl), src/CTF.cpp:98-145.
 * attr = {voltage, defocusU, defocusV, defocusTheta, Cs, amplitudeContrast,
 * phaseShift} (the field order of struct CTFAttr, include/Database.h:108-122).
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_ctf(const double* attr, double pixelSize, int N,
                      const int* iCol, const int* iRow, int K, double* out)
{
    double voltage = attr[0], dU = attr[1], dV = attr[2], theta = attr[3];
    double Cs = attr[4], A = attr[5], phaseShift = attr[6];
    double lambda = 12.2643247 / sqrt(voltage * (1 + voltage * 0.978466e-6));
    double w1 = sqrt(1 - A * A), w2 = A;
    double K1 = M_PI * lambda;
    double K2 = (M_PI / 2) * Cs * lambda * lambda * lambda;
    for (int p = 0; p < K; p++) {
        double u = hypot(iCol[p] / (pixelSize * N), iRow[p] / (pixelSize * N));
        double angle = atan2((double)iRow[p], (double)iCol[p]) - theta;
        double defocus = -(dU + dV + (dU - dV) * cos(2 * angle)) / 2;
        double u2 = u * u;
        double ki = K1 * defocus * u2 + K2 * (u2 * u2) - phaseShift;
        out[p] = -w1 * sin(ki) + w2 * cos(ki);
    }
}

/* ---------------------------------------------------------------------------
 * Log-likelihood of one hypothesis.  logDataVSPrior_m_huabin,
 * src/Optimiser.cpp:8922-8946: sum_p |X_p - c_p P_p|^2 * sigRcp_p.
 * ------------------------------------------------------------------------- */
OR_EXPORT double or_logdvp(const double* dat, const double* pri,
                           const double* ctf, const double* sigRcp, int K)
{
    double result = 0;
    for (int i = 0; i < K; i++) {
        double tr = ctf[i] * pri[2 * i], ti = ctf[i] * pri[2 * i + 1];
        double dr = dat[2 * i] - tr, di = dat[2 * i + 1] - ti;
        result += (dr * dr + di * di) * sigRcp[i];
    }
    return result;
}

/* ---------------------------------------------------------------------------
 * One local particle-filter scoring pass for one particle and one class.
 * Optimiser::updateSP, src/Optimiser.cpp:1169-1347 (no defocus search:
 * nD = 1, wD = 1): project each rotation, multiply by each phase shift,
 * score, and fold into the running-baseline marginals
 *   wC += s wR_prior(r) wT_prior(t),  wR(r) += s wC_prior wT_prior(t),
 *   wT(t) += s wC_prior wR_prior(r),  s = exp(L - baseline).
 * The weights are relative to the final baseline (the maximum L).
 * dvp (optional) receives L[r][t].
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_score_local(const double* vol, int vdim, int pf,
                              const int* iCol, const int* iRow, int K, int N,
                              const double* dat, const double* ctf,
                              const double* sigRcp,
                              const double* quat, int nR,
                              const double* trans, int nT,
                              const double* pwR, const double* pwT, double pwC,
                              double* dvp, double* wC, double* wR, double* wT,
                              double* baseLine)
{
    double* mat = (double*)malloc(sizeof(double) * 9 * (size_t)nR);
    double* tra = (double*)malloc(sizeof(double) * 2 * (size_t)nT * K);
    double* rotP = (double*)malloc(sizeof(double) * 2 * (size_t)K);
    double* allP = (double*)malloc(sizeof(double) * 2 * (size_t)K);
    or_rotmat(quat, nR, mat);
    or_translate(trans, nT, N, iCol, iRow, K, tra);
    double base = NAN, c = 0;
    for (int r = 0; r < nR; r++) wR[r] = 0;
    for (int t = 0; t < nT; t++) wT[t] = 0;
    for (int r = 0; r < nR; r++) {
        or_project(vol, vdim, mat + 9 * r, 1, iCol, iRow, K, pf, rotP);
        for (int t = 0; t < nT; t++) {
            const double* S = tra + 2 * (size_t)t * K;
            for (int p = 0; p < K; p++) {
                double a = S[2 * p], b = S[2 * p + 1];
                double e = rotP[2 * p], f = rotP[2 * p + 1];
                allP[2 * p] = a * e - b * f;
                allP[2 * p + 1] = a * f + b * e;
            }
            double w = or_logdvp(dat, allP, ctf, sigRcp, K);
            if (dvp) dvp[(size_t)r * nT + t] = w;
            if (isnan(base)) base = w;
            if (w > base) {
                double nf = exp(base - w);
                c *= nf;
                for (int i = 0; i < nR; i++) wR[i] *= nf;
                for (int i = 0; i < nT; i++) wT[i] *= nf;
                base = w;
            }
            double s = exp(w - base);
            c += s * (pwR[r] * pwT[t] * 1.0);
            wR[r] += s * (pwC * pwT[t] * 1.0);
            wT[t] += s * (pwC * pwR[r] * 1.0);
        }
    }
    *wC = c;
    *baseLine = base;
    free(mat); free(tra); free(rotP); free(allP);
}

/* ---------------------------------------------------------------------------
 * Global scan over images that share one rotation set and one translation
 * set, for class kIdx of nK.  Optimiser::doGlobalSearch,
 * src/Optimiser.cpp:759-899 (rotation-outer, translation-inner, per-image
 * running baseline), with the marginal layouts of the GPU entry point
 * ExpectGlobal3D (gpu/interface/Interface.h:221-237):
 *   wC[l*nK + k], wR[(l*nK + k)*nR + r], wT[(l*nK + k)*nT + t].
 * dat/ctf/sigRcp are image-major [nImg][K].  rotP is [nR][K] and traP
 * [nT][K] complex.  For kIdx > 0 the running baseline and the weights of the
 * earlier classes are carried in and rescaled, as the per-image baseline is
 * in the CPU scan.
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_score_global(const double* rotP, const double* traP,
                               const double* dat, const double* ctf,
                               const double* sigRcp, int nImg, int K,
                               int nR, int nT, const double* pR,
                               const double* pT, int kIdx, int nK,
                               double* wC, double* wR, double* wT,
                               double* baseL, double* dvp)
{
    double* allP = (double*)malloc(sizeof(double) * 2 * (size_t)K);
    if (kIdx == 0)
        for (int l = 0; l < nImg; l++) {
            baseL[l] = NAN;
            for (int k = 0; k < nK; k++) {
                wC[(size_t)l * nK + k] = 0;
                for (int r = 0; r < nR; r++) wR[((size_t)l * nK + k) * nR + r] = 0;
                for (int t = 0; t < nT; t++) wT[((size_t)l * nK + k) * nT + t] = 0;
            }
        }
    for (int r = 0; r < nR; r++)
        for (int t = 0; t < nT; t++) {
            const double* S = traP + 2 * (size_t)t * K;
            const double* P = rotP + 2 * (size_t)r * K;
            for (int p = 0; p < K; p++) {
                double a = S[2 * p], b = S[2 * p + 1];
                double e = P[2 * p], f = P[2 * p + 1];
                allP[2 * p] = a * e - b * f;
                allP[2 * p + 1] = a * f + b * e;
            }
            for (int l = 0; l < nImg; l++) {
                double w = or_logdvp(dat + 2 * (size_t)l * K, allP,
                                     ctf + (size_t)l * K, sigRcp + (size_t)l * K, K);
                if (dvp) dvp[((size_t)l * nR + r) * nT + t] = w;
                if (isnan(baseL[l])) baseL[l] = w;
                else if (w > baseL[l]) {
                    double offset = w - baseL[l];
                    double nf = exp(-offset);
                    for (int k = 0; k < nK; k++) {
                        wC[(size_t)l * nK + k] *= nf;
                        for (int i = 0; i < nR; i++) wR[((size_t)l * nK + k) * nR + i] *= nf;
                        for (int i = 0; i < nT; i++) wT[((size_t)l * nK + k) * nT + i] *= nf;
                    }
                    baseL[l] += offset;
                }
                double s = exp(w - baseL[l]);
                wC[(size_t)l * nK + kIdx] += s * (pR[r] * pT[t]);
                wR[((size_t)l * nK + kIdx) * nR + r] += s * pT[t];
                wT[((size_t)l * nK + kIdx) * nT + t] += s * pR[r];
            }
        }
    free(allP);
}

/* ---------------------------------------------------------------------------
 * Particle-filter narrowing and systematic resampling of one axis.
 * Particle::keepHalfHeightPeak, src/Particle.cpp:1935-1973 (applied when
 * peakFactor > 0); Particle::shuffle, src/Particle.cpp:2173-2270 (element i
 * moves to position perm[i]); Particle::resample(int, ParticleType),
 * src/Particle.cpp:1275-1463 (w *= u, normalise, cumulative sum d_cumsum
 * src/Functions/Functions.cpp:29-43, cdf /= cdf[n-1], draws u0 + j/nOut,
 * new weight 1/u of the source, PARTICLE_PRIOR_ONE include/Config.h:63);
 * Particle::normW, src/Particle.cpp:813-820.  Sums are sequential, as the
 * scalar Eigen reduction is.
 *
 * in:  u[n] likelihood weights (set by setUR/setUT), w[n] prior weights,
 *      perm[n] the shuffle permutation, u0 in [0, 1/nOut), peakFactor
 *      (<= 0 skips the narrowing), nOut.
 * out: src[nOut] index (pre-shuffle) of the source of each new sample,
 *      wOut[nOut] normalised new prior weights, *top the pre-shuffle index
 *      of the largest u after narrowing, found in shuffled order; among
 *      equal maxima the last one wins, as in gsl_sort_largest_index
 *      (GSL 2.4 sort/subsetind_source.c) behind Particle::iSort.
 * Returns 0, or -1 when the weights sum to zero.
 * ------------------------------------------------------------------------- */
OR_EXPORT int or_resample(int n, const double* uIn, const double* wIn,
                          const int* perm, double u0, double peakFactor,
                          int nOut, int* src, double* wOut, int* top)
{
    double* u = (double*)malloc(sizeof(double) * (size_t)n);
    double* w = (double*)malloc(sizeof(double) * (size_t)n);
    int* idx = (int*)malloc(sizeof(int) * (size_t)n);
    double* cdf = (double*)malloc(sizeof(double) * (size_t)n);
    int rc = 0;
    /* keepHalfHeightPeak */
    int best = 0;
    for (int i = 1; i < n; i++) if (uIn[i] > uIn[best]) best = i;
    double hh = peakFactor > 0 ? uIn[best] * peakFactor : 0;
    /* shuffle: element i goes to slot perm[i] */
    for (int i = 0; i < n; i++) {
        double ui = uIn[i];
        if (peakFactor > 0) ui = (ui < hh) ? 0 : ui - hh;
        u[perm[i]] = ui;
        w[perm[i]] = wIn[i];
        idx[perm[i]] = i;
    }
    int tb = 0;
    for (int i = 1; i < n; i++) if (u[i] >= u[tb]) tb = i;
    *top = idx[tb];
    for (int i = 0; i < n; i++) w[i] *= u[i];
    double s = w[0];
    for (int i = 1; i < n; i++) s += w[i];
    if (!(s > 0)) { rc = -1; goto done; }
    for (int i = 0; i < n; i++) w[i] /= s;
    double acc = 0;
    for (int i = 0; i < n; i++) { acc += w[i]; cdf[i] = acc; }
    double last = cdf[n - 1];
    for (int i = 0; i < n; i++) cdf[i] /= last;
    {
        int i = 0;
        for (int j = 0; j < nOut; j++) {
            double uj = u0 + j * 1.0 / nOut;
            while (uj > cdf[i]) i++;
            src[j] = idx[i];
            wOut[j] = 1.0 / u[i];
        }
    }
    s = wOut[0];
    for (int j = 1; j < nOut; j++) s += wOut[j];
    for (int j = 0; j < nOut; j++) wOut[j] /= s;
done:
    free(u); free(w); free(idx); free(cdf);
    return rc;
}

/* ---------------------------------------------------------------------------
 * Modified Kaiser-Bessel kernel table.  I0 from its power series
 * sum_k ((x/2)^k / k!)^2 (Abramowitz & Stegun 9.6.10); MKB_FT_R2,
 * src/Functions/Functions.cpp:108-126 (order 0, FUNCTIONS_MKB_ORDER_0,
 * include/Config.h:37); TabFunction::init, src/TabFunction.cpp:25-39:
 * tab[i] = f(i * b / n), i = 0..n.
 * ------------------------------------------------------------------------- */
OR_EXPORT double or_bessel_i0(double x)
{
    double q = 0.25 * x * x, term = 1, sum = 1;
    for (int k = 1; k < 200; k++) {
        term *= q / ((double)k * k);
        sum += term;
        if (term < sum * 1e-17) break;
    }
    return sum;
}

OR_EXPORT double or_mkb_ft_r2(double r2, double a, double alpha)
{
    double u2 = r2 / (a * a);
    if (u2 > 1) return 0;
    return or_bessel_i0(alpha * sqrt(1 - u2)) / or_bessel_i0(alpha);
}

OR_EXPORT void or_mkb_table(double a, double alpha, double b, int n, double* tab)
{
    double s = b / n;
    for (int i = 0; i <= n; i++) tab[i] = or_mkb_ft_r2(0 + i * s, a, alpha);
}

/* Accumulate into voxel (i, j, k), mirroring x < 0 onto the stored half
 * (Volume::addFT(Complex, int, int, int), src/Image/Volume.cpp:222-240, and
 * Volume::addFT(RFLOAT, int, int, int), :258-273). */
static inline void add_voxel(double* F, double* T, int vdim, int i, int j, int k,
                             double fr, double fi, double t)
{
    int conj = 0;
    if (i < 0) { i = -i; j = -j; k = -k; conj = 1; }
    size_t idx = vol_index(vdim, i, j, k);
    F[2 * idx] += fr;
    F[2 * idx + 1] += conj ? -fi : fi;
    T[idx] += t;
}

/* ---------------------------------------------------------------------------
 * Insertion of one weighted slice.  Reconstructor::insertP,
 * src/Reconstructor.cpp:782-863: position R (iColPad, iRowPad, 0);
 * F gets src * ctf * w, T gets ctf^2 * w (RECONSTRUCTOR_ADD_T_DURING_INSERT).
 *  kernel == 1 (MKB): Volume::addFT(value, x, y, z, a, TabFunction),
 *    src/Image/Volume.cpp:399-431 with the VOLUME_SUB_SPHERE_FT(a) box
 *    (include/Image/Volume.h:53-62): every voxel with r^2 < a^2 gets
 *    value * tab[rint(r^2 / (tabB / tabN))].
 *  kernel == 0 (trilinear): Volume::addFT(value, x, y, z),
 *    src/Image/Volume.cpp:334-369 with addFTHalf(value, w, x0), :555-640.
 * F is complex and T real, both [vdim][vdim][vdim/2+1].
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_insert(double* F, double* T, int vdim,
                         const double* img, const double* ctf,
                         const double* mat, double w,
                         const int* iColPad, const int* iRowPad, int K,
                         int kernel, double a, const double* tab,
                         double tabB, int tabN)
{
    const int half = vdim / 2;
    const double a2 = a * a, s = tabB / tabN;
    for (int p = 0; p < K; p++) {
        double c = (double)iColPad[p], r = (double)iRowPad[p];
        double x = mat[0] * c + mat[1] * r;
        double y = mat[3] * c + mat[4] * r;
        double z = mat[6] * c + mat[7] * r;
        double vr = img[2 * p] * ctf[p] * w, vi = img[2 * p + 1] * ctf[p] * w;
        double vt = ctf[p] * ctf[p] * w;
        if (kernel == 1) {
            int k0 = (int)floor(z - a), k1 = (int)ceil(z + a);
            int j0 = (int)floor(y - a), j1 = (int)ceil(y + a);
            int i0 = (int)floor(x - a), i1 = (int)ceil(x + a);
            if (k0 < -half) k0 = -half;
            if (k1 > half - 1) k1 = half - 1;
            if (j0 < -half) j0 = -half;
            if (j1 > half - 1) j1 = half - 1;
            if (i0 < -half) i0 = -half;
            if (i1 > half) i1 = half;
            for (int kk = k0; kk <= k1; kk++)
                for (int jj = j0; jj <= j1; jj++)
                    for (int ii = i0; ii <= i1; ii++) {
                        double dx = x - ii, dy = y - jj, dz = z - kk;
                        double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < a2) {
                            double kv = tab[(int)rint(r2 / s)];
                            add_voxel(F, T, vdim, ii, jj, kk, vr * kv, vi * kv, vt * kv);
                        }
                    }
        } else {
            int conj = 0;
            if (x < 0) { x = -x; y = -y; z = -z; conj = 1; }
            double xs[3] = {x, y, z}, v[3][2];
            int x0[3];
            for (int d = 0; d < 3; d++) {
                x0[d] = (int)floor(xs[d]);
                double xd = xs[d] - x0[d];
                v[d][0] = 1 - xd;
                v[d][1] = xd;
            }
            double fi = conj ? -vi : vi;
            for (int k = 0; k < 2; k++)
                for (int j = 0; j < 2; j++)
                    for (int i = 0; i < 2; i++) {
                        double ww = v[0][i] * v[1][j] * v[2][k];
                        size_t idx = vol_index(vdim, x0[0] + i, x0[1] + j, x0[2] + k);
                        F[2 * idx] += vr * ww;
                        F[2 * idx + 1] += fi * ww;
                        T[idx] += vt * ww;
                    }
        }
    }
}

/* ---------------------------------------------------------------------------
 * Fourier shell correlation between two half-FT volumes of edge vdim, shells
 * of unit width in padded-voxel radius, for r < nShell.
 * FSC(vec&, const Volume&, const Volume&), src/Functions/Spectrum.cpp:302-329.
 * ------------------------------------------------------------------------- */
OR_EXPORT void or_fsc(const double* A, const double* B, int vdim, int nShell,
                      double* fsc)
{
    double* xy = (double*)calloc((size_t)nShell, sizeof(double));
    double* xx = (double*)calloc((size_t)nShell, sizeof(double));
    double* yy = (double*)calloc((size_t)nShell, sizeof(double));
    const int nx = vdim / 2 + 1;
    for (int z = 0; z < vdim; z++)
        for (int y = 0; y < vdim; y++)
            for (int x = 0; x < nx; x++) {
                int fz = z < vdim / 2 ? z : z - vdim, fy = y < vdim / 2 ? y : y - vdim;
                int u = (int)rint(sqrt((double)x * x + (double)fy * fy + (double)fz * fz));
                if (u >= nShell) continue;
                size_t i = ((size_t)z * vdim + y) * nx + x;
                double ar = A[2 * i], ai = A[2 * i + 1], br = B[2 * i], bi = B[2 * i + 1];
                xy[u] += ar * br + ai * bi;
                xx[u] += ar * ar + ai * ai;
                yy[u] += br * br + bi * bi;
            }
    for (int u = 0; u < nShell; u++)
        fsc[u] = (xx[u] * yy[u] == 0) ? 0.0 : xy[u] / sqrt(xx[u] * yy[u]);
    free(xy); free(xx); free(yy);
}


/* ---------------------------------------------------------------------------
 * Symmetrisation of a half transform.  SYMMETRIZE_FT (include/Geometry/
 * Transformation.h:170-196): the result is the volume plus, for every
 * symmetry element R, the volume transformed by R -- VOL_TRANSFORM_MAT_FT
 * (:104-125), whose voxel v = (i, j, k) of the half grid (i >= 0) holds the
 * original sampled trilinearly at R v (getByInterpolationFT, LINEAR_INTERP:
 * the Friedel mate conjugated for a negative x) when |R v|^2 < r^2, else 0.
 * vol complex [vdim][vdim][vdim/2 + 1], in place; mats [nSym][9] row-major.
 */
void or_symmetrize(double* vol, int vdim, const double* mats, int nSym, double r)
{
    const int nx = vdim / 2 + 1, half = vdim / 2;
    const size_t n = (size_t)vdim * vdim * nx;
    double* src = (double*)malloc(sizeof(double) * 2 * n);
    memcpy(src, vol, sizeof(double) * 2 * n);
    for (int s = 0; s < nSym; s++) {
        const double* m = mats + 9 * s;
        for (int z = 0; z < vdim; z++) {
            const int k = z < half ? z : z - vdim;
            for (int y = 0; y < vdim; y++) {
                const int j = y < half ? y : y - vdim;
                for (int i = 0; i < nx; i++) {
                    const double a = m[0] * i + m[1] * j + m[2] * k;
                    const double b = m[3] * i + m[4] * j + m[5] * k;
                    const double c = m[6] * i + m[7] * j + m[8] * k;
                    if (a * a + b * b + c * c < r * r) {
                        double out[2];
                        sample_trilinear(src, vdim, a, b, c, out);
                        const size_t idx = ((size_t)z * vdim + y) * nx + i;
                        vol[2 * idx] += out[0];
                        vol[2 * idx + 1] += out[1];
                    }
                }
            }
        }
    }
    free(src);
}
