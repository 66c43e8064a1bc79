"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE, NOT PRODUCT.

Loads oracle/liboracle.so (the double-precision restatement in
tg3_oracle.c, built on demand with gcc) and, where it exists,
oracle/_ref/libthunder_ref.so (the reference's own sources compiled by
oracle/ref/Makefile).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline / reference arm use this module.

Every wrapper takes and returns numpy arrays; complex arrays are numpy
complex128 (interleaved doubles in C).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libthunder_ref.so"


def _default_ref_tree() -> str:
    """The THUNDER tree the cross-check library is built from: THUNDER_REF,
    else a tree named `reference` beside the repository's folder (the build
    recipe's default too)."""
    if os.environ.get("THUNDER_REF"):
        return os.environ["THUNDER_REF"]
    return str(HERE.parent.parent / "reference")


REF_TREE = Path(_default_ref_tree())

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_c128p = np.ctypeslib.ndpointer(dtype=np.complex128, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_c = ctypes.c_int
_d = ctypes.c_double


def build(force: bool = False) -> Path:
    """Compile tg3_oracle.c into liboracle.so (gcc, -O2, portable flags)."""
    src = HERE / "tg3_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        # no contraction into fused multiply-adds: the same double rounding on
        # every machine (gcc contracts by default where the target has FMA),
        # as the reference's x86 build without FMA computes
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-fno-fast-math", "-ffp-contract=off",
                        "-o", str(LIB), str(src), "-lm"], check=True)
    return LIB


def build_ref() -> Path | None:
    """Compile the reference cross-check library when the THUNDER tree is
    present (never on a machine without it).  Returns its path or None."""
    if not (REF_TREE / "src" / "Projector.cpp").exists():
        return REF_LIB if REF_LIB.exists() else None
    subprocess.run(["make", "-s", "-j8", "-C", str(HERE / "ref"), f"REF={REF_TREE}"],
                   check=True, stdout=subprocess.DEVNULL)
    return REF_LIB


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(str(build()))
        L.or_pixel_index.argtypes = [_c, _d, _d, _i32p, _i32p, _i32p, _i32p, _c]
        L.or_pixel_index.restype = _c
        L.or_rotmat.argtypes = [_f64p, _c, _f64p]
        L.or_project.argtypes = [_c128p, _c, _f64p, _c, _i32p, _i32p, _c, _c, _c128p]
        L.or_project2d.argtypes = [_c128p, _c, _f64p, _c, _i32p, _i32p, _c, _c, _c128p]
        L.or_insert2d.argtypes = [_c128p, _f64p, _c, _c128p, _f64p, _d, _d, _d, _i32p, _i32p, _c]
        L.or_translate.argtypes = [_f64p, _c, _c, _i32p, _i32p, _c, _c128p]
        L.or_translate_image.argtypes = [_c128p, _d, _d, _c, _i32p, _i32p, _c, _c128p]
        L.or_ctf.argtypes = [_f64p, _d, _c, _i32p, _i32p, _c, _f64p]
        L.or_logdvp.argtypes = [_c128p, _c128p, _f64p, _f64p, _c]
        L.or_logdvp.restype = _d
        L.or_score_local.argtypes = [_c128p, _c, _c, _i32p, _i32p, _c, _c,
                                     _c128p, _f64p, _f64p, _f64p, _c, _f64p, _c,
                                     _f64p, _f64p, _d,
                                     ctypes.c_void_p, ctypes.c_void_p, _f64p, _f64p,
                                     ctypes.c_void_p]
        L.or_score_global.argtypes = [_c128p, _c128p, _c128p, _f64p, _f64p, _c, _c,
                                      _c, _c, _f64p, _f64p, _c, _c, _f64p, _f64p,
                                      _f64p, _f64p, ctypes.c_void_p]
        L.or_resample.argtypes = [_c, _f64p, _f64p, _i32p, _d, _d, _c, _i32p,
                                  _f64p, ctypes.POINTER(_c)]
        L.or_resample.restype = _c
        L.or_bessel_i0.argtypes = [_d]
        L.or_bessel_i0.restype = _d
        L.or_mkb_table.argtypes = [_d, _d, _d, _c, _f64p]
        L.or_insert.argtypes = [_c128p, _f64p, _c, _c128p, _f64p, _f64p, _d,
                                _i32p, _i32p, _c, _c, _d, _f64p, _d, _c]
        L.or_fsc.argtypes = [_c128p, _c128p, _c, _c, _f64p]
        L.or_symmetrize.argtypes = [_c128p, _c, _f64p, _c, _d]
        _lib = L
    return _lib


def ref():
    """The compiled reference cross-check library, or None if unavailable."""
    global _ref
    if _ref is None:
        path = REF_LIB if REF_LIB.exists() else build_ref()
        if path is None or not Path(path).exists():
            return None
        R = ctypes.CDLL(str(path), mode=os.RTLD_LAZY)
        R.ref_rotmat.argtypes = [_f64p, _c, _f64p]
        R.ref_project.argtypes = [_c128p, _c, _f64p, _c, _i32p, _i32p, _c, _c, _c128p]
        R.ref_project2d.argtypes = [_c128p, _c, _f64p, _c, _i32p, _i32p, _c, _c, _c128p]
        R.ref_insert2d.argtypes = [_c128p, _f64p, _c, _c128p, _f64p, _d, _d, _d, _i32p, _i32p, _c]
        R.ref_read_mrc.argtypes = [ctypes.c_char_p, _c, _c, _f64p]
        R.ref_read_mrc.restype = _c
        R.ref_prep_image.argtypes = [_f64p, _c, _d, _c, _f64p, _f64p]
        R.ref_power_spectrum.argtypes = [_c128p, _c, _c, _f64p]
        R.ref_translate.argtypes = [_f64p, _c, _c, _i32p, _i32p, _c, _c128p]
        R.ref_translate_image.argtypes = [_c128p, _d, _d, _c, _i32p, _i32p, _c, _c128p]
        R.ref_ctf.argtypes = [_f64p, _d, _c, _i32p, _i32p, _c, _f64p]
        R.ref_logdvp.argtypes = [_c128p, _c128p, _f64p, _f64p, _c]
        R.ref_logdvp.restype = _d
        R.ref_logdvp_mn.argtypes = [_c128p, _c128p, _f64p, _f64p, _c, _c, _f64p]
        R.ref_mkb_table.argtypes = [_d, _d, _d, _c, _f64p]
        R.ref_insert.argtypes = [_c128p, _f64p, _c, _c128p, _f64p, _f64p, _d,
                                 _i32p, _i32p, _c, _c, _d, _d, _d, _c]
        R.ref_resample.argtypes = [_c, _f64p, _f64p, _u64p, _d, _c, _c, _i32p, _f64p]
        R.ref_resample.restype = _d
        R.ref_sort_descend.argtypes = [_f64p, _c, _u64p]
        R.ref_symmetrize.argtypes = [_c128p, _c, _f64p, _c, _d]
        R.ref_reconstruct.argtypes = [_c, _c, _c, _d, _d, _c, _c128p, _f64p, _f64p, _c,
                                      _c, _c, _c, _f64p]
        R.ref_reconstruct.restype = _c
        R.ref_fw_image.argtypes = [_f64p, _c, _c128p]
        R.ref_remask.argtypes = [_c128p, _c, _d, _d]
        _ref = R
    return _ref


def _a(x, dt):
    return np.ascontiguousarray(x, dtype=dt)


# ----------------------------------------------------------------------------
# oracle wrappers (liboracle)
# ----------------------------------------------------------------------------
def pixel_index(size, rU, rL):
    n = (int(rU) + 3) * (2 * int(rU) + 4)
    out = [np.zeros(n, np.int32) for _ in range(4)]
    K = lib().or_pixel_index(size, float(rU), float(rL), *out, n)
    return tuple(o[:K] for o in out)


def rotmat(quat):
    q = _a(quat, np.float64).reshape(-1, 4)
    m = np.zeros((len(q), 9))
    lib().or_rotmat(q, len(q), m)
    return m.reshape(-1, 3, 3)


def project(vol, mat, iCol, iRow, pf):
    vol = _a(vol, np.complex128)
    mat = _a(mat, np.float64).reshape(-1, 9)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    out = np.zeros((len(mat), len(iCol)), np.complex128)
    lib().or_project(vol, vol.shape[0], mat, len(mat), iCol, iRow, len(iCol), pf, out)
    return out


def project2d(img, rot, iCol, iRow, pf):
    """2-D projections of a half transform img [vdim][vdim/2 + 1] at in-plane
    rotations rot [nR][2] = (cos, sin); [nR][K] complex."""
    img = _a(img, np.complex128)
    rot = _a(rot, np.float64).reshape(-1, 2)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    out = np.zeros((len(rot), len(iCol)), np.complex128)
    lib().or_project2d(img, img.shape[0], rot, len(rot), iCol, iRow, len(iCol), pf, out)
    return out


def insert2d(F, T, img, c, rot, w, iColPad, iRowPad):
    """Add one slice into a 2-D F (complex) and T (real) in place."""
    lib().or_insert2d(F, T, F.shape[0], _a(img, np.complex128), _a(c, np.float64),
                      float(rot[0]), float(rot[1]), float(w), _a(iColPad, np.int32),
                      _a(iRowPad, np.int32), len(iColPad))


def translate(trans, N, iCol, iRow):
    trans = _a(trans, np.float64).reshape(-1, 2)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    out = np.zeros((len(trans), len(iCol)), np.complex128)
    lib().or_translate(trans, len(trans), N, iCol, iRow, len(iCol), out)
    return out


def translate_image(img, tx, ty, N, iCol, iRow):
    img = _a(img, np.complex128)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    out = np.zeros_like(img)
    lib().or_translate_image(img, tx, ty, N, iCol, iRow, len(iCol), out)
    return out


def ctf(attr, pixel_size, N, iCol, iRow):
    attr = _a(attr, np.float64).reshape(-1, 7)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    out = np.zeros((len(attr), len(iCol)))
    for i in range(len(attr)):
        row = np.zeros(len(iCol))
        lib().or_ctf(_a(attr[i], np.float64), pixel_size, N, iCol, iRow, len(iCol), row)
        out[i] = row
    return out


def logdvp(dat, pri, c, sigRcp):
    return lib().or_logdvp(_a(dat, np.complex128), _a(pri, np.complex128),
                           _a(c, np.float64), _a(sigRcp, np.float64), len(c))


def score_local(vol, pf, iCol, iRow, N, dat, c, sigRcp, quat, trans, pwR, pwT,
                pwC=1.0, want_dvp=True):
    """One particle's local scan.  Returns dict(dvp [nR, nT], wC, wR, wT, base)."""
    vol = _a(vol, np.complex128)
    iCol, iRow = _a(iCol, np.int32), _a(iRow, np.int32)
    quat = _a(quat, np.float64).reshape(-1, 4)
    trans = _a(trans, np.float64).reshape(-1, 2)
    nR, nT = len(quat), len(trans)
    dvp = np.zeros((nR, nT)) if want_dvp else None
    wC = np.zeros(1)
    wR = np.zeros(nR)
    wT = np.zeros(nT)
    base = np.zeros(1)
    lib().or_score_local(vol, vol.shape[0], pf, iCol, iRow, len(iCol), N,
                         _a(dat, np.complex128), _a(c, np.float64),
                         _a(sigRcp, np.float64), quat, nR, trans, nT,
                         _a(pwR, np.float64), _a(pwT, np.float64), float(pwC),
                         dvp.ctypes.data if want_dvp else None,
                         wC.ctypes.data, wR, wT, base.ctypes.data)
    return dict(dvp=dvp, wC=wC[0], wR=wR, wT=wT, base=base[0])


def score_global(rotP, traP, dat, c, sigRcp, pR, pT, kIdx=0, nK=1, state=None,
                 want_dvp=True):
    """Global scan of nImg images over shared rotation/translation banks.
    `state` (wC, wR, wT, baseL) carries earlier classes' results."""
    rotP, traP = _a(rotP, np.complex128), _a(traP, np.complex128)
    dat = _a(dat, np.complex128)
    nImg, K = dat.shape
    nR, nT = rotP.shape[0], traP.shape[0]
    if state is None:
        state = (np.zeros(nImg * nK), np.zeros(nImg * nK * nR),
                 np.zeros(nImg * nK * nT), np.zeros(nImg))
    wC, wR, wT, baseL = state
    dvp = np.zeros((nImg, nR, nT)) if want_dvp else None
    lib().or_score_global(rotP, traP, dat, _a(c, np.float64), _a(sigRcp, np.float64),
                          nImg, K, nR, nT, _a(pR, np.float64), _a(pT, np.float64),
                          kIdx, nK, wC, wR, wT, baseL,
                          dvp.ctypes.data if want_dvp else None)
    return dict(wC=wC, wR=wR, wT=wT, baseL=baseL, dvp=dvp)


def resample(u, w, perm, u0, peak_factor, n_out):
    u, w = _a(u, np.float64), _a(w, np.float64)
    perm = _a(perm, np.int32)
    src = np.zeros(n_out, np.int32)
    wout = np.zeros(n_out)
    top = ctypes.c_int(0)
    rc = lib().or_resample(len(u), u, w, perm, float(u0), float(peak_factor),
                           n_out, src, wout, ctypes.byref(top))
    if rc != 0:
        raise ValueError("weights sum to zero")
    return src, wout, top.value


def peak_factor_r(u):
    """Particle::setPeakFactor(PAR_R) in 3D (src/Particle.cpp:1886-1896):
    clamp(u_(n/8) / u_(0), 1e-3, 0.5) over the descending order of u."""
    u = np.asarray(u, np.float64)
    order = descend_order(u)
    return max(1e-3, min(0.5, u[order[len(u) // 8]] / u[order[0]]))


def descend_order(v):
    """Indices of v in descending order, equal values ordered last-index
    first, as gsl_sort_largest_index produces them (GSL 2.4,
    sort/subsetind_source.c) for d_index_sort_descend
    (src/Functions/Functions.cpp:72-79)."""
    v = np.asarray(v)
    n = len(v)
    return np.lexsort((-np.arange(n), -v))


def mkb_table(a, alpha, b, n):
    tab = np.zeros(n + 1)
    lib().or_mkb_table(a, alpha, b, n, tab)
    return tab


def bessel_i0(x):
    return lib().or_bessel_i0(float(x))


def insert(F, T, img, c, mat, w, iColPad, iRowPad, kernel, a, tab, tabB):
    """Accumulate one slice into F (complex) and T (real), in place."""
    vdim = F.shape[0]
    lib().or_insert(F, T, vdim, _a(img, np.complex128), _a(c, np.float64),
                    _a(mat, np.float64).reshape(9), float(w),
                    _a(iColPad, np.int32), _a(iRowPad, np.int32), len(iColPad),
                    int(kernel), float(a), _a(tab, np.float64), float(tabB),
                    len(tab) - 1)


def fsc(A, B, n_shell):
    A, B = _a(A, np.complex128), _a(B, np.complex128)
    out = np.zeros(n_shell)
    lib().or_fsc(A, B, A.shape[0], n_shell, out)
    return out


def symmetrize(vol, mats, r):
    """SYMMETRIZE_FT of a half transform vol [vdim][vdim][vdim/2 + 1]
    (complex; a real T as its real part) over the symmetry elements mats
    [nSym][3][3] within radius r; returns a new array."""
    v = np.array(vol, dtype=np.complex128, order="C")
    m = _a(mats, np.float64).reshape(-1, 9)
    lib().or_symmetrize(v, v.shape[0], m, len(m), float(r))
    return v


def ref_symmetrize(vol, mats, r):
    """The same through the compiled reference (None if unavailable)."""
    R = ref()
    if R is None:
        return None
    v = np.array(vol, dtype=np.complex128, order="C")
    m = _a(mats, np.float64).reshape(-1, 9)
    R.ref_symmetrize(v, v.shape[0], m, len(m), float(r))
    return v


def ref_reconstruct(F, T, pf, max_radius, fsc, join_half=False, grid_corr=True, a=1.9,
                    alpha=15.0, n_thread=1):
    """Reconstructor::reconstruct through the compiled reference (None if
    unavailable): F complex, T real on the padded half grid ((vdim,) * (d - 1)
    + (vdim/2 + 1,)), d = 2 or 3 -> the N^d map, coordinate i at index
    i + N/2.  The reference's build configures the trilinear real-space
    correction."""
    R = ref()
    if R is None:
        return None
    F = _a(F, np.complex128)
    T = _a(T, np.float64)
    dim, vdim = F.ndim, F.shape[0]
    N = vdim // pf
    f = _a(np.zeros(1) if fsc is None else fsc, np.float64)
    out = np.zeros((N,) * dim)
    rc = R.ref_reconstruct(dim, N, pf, float(a), float(alpha), int(max_radius), F, T, f,
                           len(f), int(join_half), int(grid_corr), int(n_thread), out.reshape(-1))
    if rc != 0:
        raise ValueError("reference reconstruct: accumulator size mismatch")
    return out


def ref_fw_image(img):
    """FFT::fw of one N x N image in the Image's storage order (centre at
    index 0) through the compiled reference and its FFTW (None if
    unavailable) -> the half transform (N, N/2 + 1)."""
    R = ref()
    if R is None:
        return None
    img = _a(img, np.float64)
    N = img.shape[0]
    out = np.zeros((N, N // 2 + 1), np.complex128)
    R.ref_fw_image(img.reshape(-1), N, out)
    return out


def ref_remask(F, r, ew=6.0):
    """Optimiser::reMaskImg of one half transform F (N, N/2 + 1) through the
    compiled reference (None if unavailable)."""
    R = ref()
    if R is None:
        return None
    F = np.array(F, dtype=np.complex128, order="C")
    R.ref_remask(F, F.shape[0], float(r), float(ew))
    return F
