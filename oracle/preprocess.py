"""Oracle (test infrastructure only): the reference's image preprocessing in
numpy, float64 -- the checker for tg3_prepare_images_d, never on the product
path.  Pinned against the compiled reference's bgMeanStddev / bgStddev /
softMask and ImageFile reader (tests/test_oracle_pin.py); the transform is
FFTW's unnormalised forward r2c (src/FFT.cpp:118-140), here numpy's rfft2.

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
