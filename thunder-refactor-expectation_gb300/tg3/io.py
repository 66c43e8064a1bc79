"""MRC stacks and .thu particle databases through the library's readers and
writers (src/Image/ImageFile.cpp, src/Database.cpp), as numpy arrays."""
from __future__ import annotations

import ctypes

import numpy as np

from . import check, lib, ptr

THU_COLUMNS = 27
THU_PATH, THU_MICROGRAPH, THU_GROUP, THU_CLASS = 7, 8, 11, 12
# the reference's column names (include/Database.h), by index
THU_FIELDS = ("voltage", "defocusU", "defocusV", "defocusTheta", "Cs", "amplitudeContrast",
              "phaseShift", "path", "micrographPath", "coordX", "coordY", "groupID", "classID",
              "q0", "q1", "q2", "q3", "k1", "k2", "k3", "tx", "ty", "stdTx", "stdTy",
              "defocusFactor", "stdDefocusFactor", "score")


def spectrum_pixels(N, r):
    """The half-transform pixels of shells rint(|k|) < r, in the order of the
    reference's powerSpectrum loop (rows j in [-N/2, N/2), columns i in
    [0, N/2]): iCol, iRow (int32)."""
    j, i = np.meshgrid(np.arange(-N // 2, N // 2), np.arange(N // 2 + 1), indexing="ij")
    i, j = i.ravel(), j.ravel()
    q = i * i + j * j
    keep = (q < r * r) & (np.rint(np.sqrt(q)) < r)
    return i[keep].astype(np.int32), j[keep].astype(np.int32)


def mrc_info(path):
    """(nx, ny, nz, mode, pixel size) of an MRC file."""
    v = [ctypes.c_int() for _ in range(4)]
    px = ctypes.c_float()
    check(lib().tg3_mrc_info(str(path).encode(), *[ctypes.byref(x) for x in v],
                             ctypes.byref(px)))
    return tuple(x.value for x in v) + (px.value,)


def read_mrc(path, first=0, count=None):
    """Sections [first, first + count) as float32 (count, ny, nx), file order."""
    nx, ny, nz, _, _ = mrc_info(path)
    count = nz - first if count is None else count
    out = np.empty((count, ny, nx), np.float32)
    check(lib().tg3_mrc_read(str(path).encode(), first, count, ptr(out)))
    return out


def write_mrc(path, data, pixel_size=1.0, volume=False):
    """float32 stack or volume (nz, ny, nx) in file order."""
    a = np.ascontiguousarray(data, np.float32)
    if a.ndim == 2:
        a = a[None]
    nz, ny, nx = a.shape
    check(lib().tg3_mrc_write(str(path).encode(), ptr(a), nx, ny, nz, float(pixel_size),
                              int(volume)))


def centred(img):
    """The reference's in-memory layout of an image read from a file: the
    centre pixel (N/2, N/2) at index 0 (ImageFile's MESH_IMAGE_INDEX)."""
    return np.fft.ifftshift(img, axes=(-2, -1))


def read_thu(path, stride=1024):
    """cols (n, 27) float64 (path columns NaN), particle paths, micrograph paths."""
    n = ctypes.c_int()
    check(lib().tg3_thu_count(str(path).encode(), ctypes.byref(n)))
    n = n.value
    cols = np.empty((n, THU_COLUMNS))
    p = np.zeros((n, stride), np.uint8)
    m = np.zeros((n, stride), np.uint8)
    check(lib().tg3_thu_read(str(path).encode(), n, ptr(cols), ptr(p), ptr(m), stride))
    dec = lambda a: [bytes(r[:np.argmin(r)] if 0 in r else r).decode() for r in a]
    return cols, dec(p), dec(m)


def write_thu(path, cols, paths, micrographs, stride=1024):
    cols = np.ascontiguousarray(cols, np.float64)
    n = cols.shape[0]
    if cols.shape != (n, THU_COLUMNS) or len(paths) != n or len(micrographs) != n:
        raise ValueError("cols must be (n, 27) with n paths and n micrograph paths")

    def enc(strs):
        a = np.zeros((n, stride), np.uint8)
        for i, s in enumerate(strs):
            b = s.encode()
            if len(b) >= stride:
                raise ValueError("path longer than the stride")
            a[i, :len(b)] = np.frombuffer(b, np.uint8)
        return a

    p, m = enc(paths), enc(micrographs)
    check(lib().tg3_thu_write(str(path).encode(), n, ptr(cols), ptr(p), ptr(m), stride))
