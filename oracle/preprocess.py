"""Oracle (test infrastructure only): the reference's image preprocessing in
numpy, float64 -- the checker for tg3_prepare_images_d, never on the product
path.  Pinned against the compiled reference's bgMeanStddev / bgStddev /
softMask and ImageFile reader, and, through the reference's FFT class on the
vendored FFTW, the whole chain with its transform and the re-mask
(tests/test_formats_cpu.py live, tests/test_oracle_golden.py on fixtures).
The transform is FFTW's unnormalised forward r2c (src/FFT.cpp:118-140),
here numpy's rfft2.

Steps (src/Optimiser.cpp): substractBgImg :4917 (background outside radius r
about the file's pixel (N/2, N/2): mean and n - 1 deviation, subtracted and
divided; bgMeanStddev, src/Image/ImageFunctions.cpp:607-620), statImg :4796
(stdN = mean over images of the normalised background deviation about 0;
bgStddev, ImageFunctions.cpp:585-596), maskImg :4953 with zeroMask
(softMask, src/Functions/Mask.cpp:363-385, edge EDGE_WIDTH_RL = 6),
normaliseImg :4987 (1 / stdN), fwImg :5003 on the image held with its centre
at index 0 (MESH_IMAGE_INDEX of include/Image/ImageFile.h), allocPreCal
:7995-8030 (pixels at (iCol, iRow mod N))."""
from __future__ import annotations

import numpy as np

EDGE_WIDTH_RL = 6.0


def centred_coords(N):
    c = np.arange(N) - N // 2
    return np.meshgrid(c, c)          # (i: column, j: row), file order


def normalise(img, r):
    """(x - m) / s and the statistics (m, s, sN) of one file-order image."""
    i, j = centred_coords(img.shape[-1])
    bg = (i * i + j * j) > r * r
    v = img[bg].astype(np.float64)
    m = v.mean()
    s = np.sqrt(((v - m) ** 2).sum() / (v.size - 1))
    y = (img - m) / s
    sn = np.sqrt((y[bg] ** 2).sum() / (v.size - 1))
    return y, (m, s, sn)


def soft_mask(y, r, ew=EDGE_WIDTH_RL):
    i, j = centred_coords(y.shape[-1])
    u = np.sqrt(i * i + j * j)
    w = 0.5 - 0.5 * np.cos((u - r) / ew * np.pi)
    out = np.where(u < r, y, y * (1 - w))
    return np.where(u > r + ew, 0.0, out)


def preprocess(imgs, r, iCol, iRow, mask=True, std_n=None):
    """imgs (n, N, N) file order -> dat (n, K) complex128, stats (n, 3),
    and the transformed-from images (n, N, N) with their centre at index 0."""
    imgs = np.asarray(imgs, np.float64)
    n, N, _ = imgs.shape
    ys, st = [], []
    for l in range(n):
        y, s = normalise(imgs[l], r)
        ys.append(y)
        st.append(s)
    st = np.array(st)
    stdN = float(std_n) if std_n else st[:, 2].mean()
    real = np.stack([(soft_mask(y, r) if mask else y) / stdN for y in ys])
    corner = np.fft.ifftshift(real, axes=(-2, -1))
    F = np.fft.rfft2(corner)
    rows = np.asarray(iRow) % N
    dat = F[:, rows, np.asarray(iCol)]
    return dat, st, corner


def power_spectrum(F, r):
    """Shell means of |F|^2 over a half transform F (N, N/2 + 1), rows j in
    wrapped order: shells u = rint(|k|) < r among pixels with i^2 + j^2 < r^2
    (powerSpectrum, src/Functions/Spectrum.cpp:161-190)."""
    N = F.shape[0]
    j, i = np.meshgrid(np.arange(-N // 2, N // 2), np.arange(N // 2 + 1), indexing="ij")
    q = i * i + j * j
    u = np.rint(np.sqrt(q)).astype(int)
    keep = (q < r * r) & (u < r)
    vals = np.abs(F[j[keep] % N, i[keep]]) ** 2
    s = np.bincount(u[keep], weights=vals, minlength=r)[:r]
    c = np.bincount(u[keep], minlength=r)[:r]
    return s / c


def sigma(models, datM, datN, offsets, iCol, iRow, N, r, groups, n_group, by_group, mask_radius,
          pixel_size):
    """Optimiser::allReduceSigma (src/Optimiser.cpp:6355-6630, rank-1 pose,
    whole frequency range) over pixel data at the pixels (iCol, iRow) of the
    shells below r: models [n][K] = ctf P(R) S(t) of each image's best pose;
    the unmasked model is that times S(-offset).  Returns sig, sigRcp
    [n_group][r]."""
    iCol, iRow = np.asarray(iCol), np.asarray(iRow)
    u = np.rint(np.sqrt(iCol * iCol + iRow * iRow)).astype(int)
    cnt = np.bincount(u, minlength=r)[:r]
    shell = lambda v: np.bincount(u, weights=v, minlength=r)[:r] / cnt
    acc = np.zeros((n_group, 3 * r + 1))
    for l in range(len(models)):
        M = models[l]
        ox, oy = (offsets[l] if offsets is not None else (0.0, 0.0))
        Nm = M * np.exp(2j * np.pi * (iCol * ox + iRow * oy) / N)
        g = groups[l] - 1 if by_group else 0
        acc[g, :r] += shell(np.abs(datM[l] - M) ** 2) / 2
        acc[g, r:2 * r] += shell(np.abs(datN[l] - Nm) ** 2) / 2
        acc[g, 2 * r:3 * r] += np.sqrt(shell(np.abs(M) ** 2) / shell(np.abs(datM[l]) ** 2))
        acc[g, 3 * r] += 1
    if not by_group:
        acc[:] = acc[0]
    w = acc[:, 3 * r:3 * r + 1]
    sM, sN, svd = acc[:, :r] / w, acc[:, r:2 * r] / w, acc[:, 2 * r:3 * r] / w
    alpha = np.sqrt(np.pi * (mask_radius / (N * pixel_size)) ** 2)
    ratio = np.minimum(1.0, svd)
    sig = ratio * sM + (1 - ratio) * alpha * sN
    return sig, -0.5 / sig


def remask(F, r, ew=EDGE_WIDTH_RL):
    """Optimiser::reMaskImg (src/Optimiser.cpp:6053-6111; on the GPU reMask,
    gpu/src/cuthunder.cu:9384-9560): every half transform F [n][N][N/2 + 1]
    (the image's centre at index 0) taken to real space by the normalised
    inverse transform (FFT::bw, src/FFT.cpp:143-167), multiplied by the soft
    mask of radius r and edge ew about the centre, and transformed back by
    the unnormalised forward transform."""
    F = np.asarray(F, np.complex128)
    N = F.shape[-2]
    real = np.fft.irfft2(F, s=(N, N))
    masked = np.stack([np.fft.ifftshift(soft_mask(np.fft.fftshift(x), r, ew)) for x in real])
    return np.fft.rfft2(masked)
