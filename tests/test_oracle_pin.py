"""Live pin: the oracle restatement against the reference's own compiled
sources (oracle/_ref, built from the THUNDER tree by oracle/ref/Makefile) on
fresh seeded cases.  Skipped where the THUNDER tree is absent; the golden
fixtures cover those machines."""
import numpy as np
import pytest

from oracle import oracle as O
from tg3 import synth

R = O.ref()
pytestmark = pytest.mark.skipif(R is None, reason="reference sources unavailable")


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(7)
    box, pf = 24, 2
    iCol, iRow, _, _ = synth.pixel_index(box, 10, 1)
    bm = synth.blob_map(rng, 12, (2.0, 4.0), 1.5, 7.0)
    vol = np.ascontiguousarray(synth.padded_volume(bm, box, pf).numpy())
    return dict(rng=rng, box=box, pf=pf, iCol=iCol, iRow=iRow, vol=vol, K=len(iCol))


def test_project(case):
    rng = case["rng"]
    q = synth.haar_quaternions(rng, 64)
    m = np.zeros((64, 9))
    R.ref_rotmat(q, 64, m)
    P2 = np.zeros((64, case["K"]), np.complex128)
    R.ref_project(case["vol"], case["vol"].shape[0], m, 64, case["iCol"], case["iRow"],
                  case["K"], case["pf"], P2)
    P1 = O.project(case["vol"], O.rotmat(q), case["iCol"], case["iRow"], case["pf"])
    assert np.array_equal(P1, P2)


def test_insert_mkb(case):
    rng = case["rng"]
    K, pf = case["K"], case["pf"]
    q = synth.haar_quaternions(rng, 3)
    tab = O.mkb_table(1.9, 15.0, (pf * 1.9) ** 2, 100000)
    F1 = np.zeros(case["vol"].shape, np.complex128)
    T1 = np.zeros(case["vol"].shape)
    F2, T2 = F1.copy(), T1.copy()
    m = O.rotmat(q)
    for s in range(3):
        img = rng.standard_normal(K) + 1j * rng.standard_normal(K)
        c = rng.standard_normal(K)
        O.insert(F1, T1, img, c, m[s], 0.5, case["iCol"] * pf, case["iRow"] * pf, 1,
                 pf * 1.9, tab, (pf * 1.9) ** 2)
        R.ref_insert(F2, T2, F2.shape[0], img, c, np.ascontiguousarray(m[s].ravel()), 0.5,
                     (case["iCol"] * pf).astype(np.int32), (case["iRow"] * pf).astype(np.int32),
                     K, 1, 1.9, 15.0, (pf * 1.9) ** 2, 100000)
    np.testing.assert_allclose(F1, F2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(T1, T2, rtol=0, atol=1e-12)


@pytest.mark.parametrize("n,n_out,mode", [(7, 7, 0), (300, 250, 1), (2000, 2000, 1)])
def test_resample(n, n_out, mode):
    rng = np.random.default_rng(n)
    u = np.exp(2 * rng.standard_normal(n))
    w = rng.random(n)
    perm = rng.permutation(n)
    u0 = rng.random() / n_out
    src2 = np.zeros(n_out, np.int32)
    w2 = np.zeros(n_out)
    R.ref_resample(n, u, w, perm.astype(np.uint64), u0, n_out, mode, src2, w2)
    pfac = O.peak_factor_r(u) if mode else 0.0
    src1, w1, _ = O.resample(u, w, perm.astype(np.int32), u0, pfac, n_out)
    assert np.array_equal(src1, src2)
    assert np.array_equal(w1, w2)


def test_project2d():
    """The 2-D projection (bilinear in a half transform, Friedel mirror,
    wrapped rows) against the reference's Image::getByInterpolationFT."""
    rng = np.random.default_rng(17)
    box, pf = 24, 2
    vdim = box * pf
    iCol, iRow, _, _ = synth.pixel_index(box, 10, 1)
    img = np.ascontiguousarray(rng.standard_normal((vdim, vdim // 2 + 1)) +
                               1j * rng.standard_normal((vdim, vdim // 2 + 1)))
    ang = rng.uniform(0, 2 * np.pi, 40)
    rot = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    P2 = np.zeros((40, len(iCol)), np.complex128)
    R.ref_project2d(img, vdim, rot, 40, iCol, iRow, len(iCol), pf, P2)
    P1 = O.project2d(img, rot, iCol, iRow, pf)
    np.testing.assert_allclose(P1, P2, rtol=0, atol=1e-12)


def test_insert2d():
    """The 2-D insertion (bilinear into a half transform, Friedel mirror,
    wrapped rows) against the reference's Image::addFT, complex and real."""
    rng = np.random.default_rng(19)
    box, pf = 24, 2
    vdim = box * pf
    iCol, iRow, _, _ = synth.pixel_index(box, 10, 1)
    K = len(iCol)
    ic, ir = np.ascontiguousarray(iCol * pf, np.int32), np.ascontiguousarray(iRow * pf, np.int32)
    F1 = np.zeros((vdim, vdim // 2 + 1), np.complex128)
    T1 = np.zeros((vdim, vdim // 2 + 1))
    F2, T2 = F1.copy(), T1.copy()
    for ang in rng.uniform(0, 2 * np.pi, 6):
        img = rng.standard_normal(K) + 1j * rng.standard_normal(K)
        c = rng.uniform(-1, 1, K)
        w = float(rng.uniform(0.1, 1))
        O.insert2d(F1, T1, img, c, (np.cos(ang), np.sin(ang)), w, ic, ir)
        R.ref_insert2d(F2, T2, vdim, np.ascontiguousarray(img), np.ascontiguousarray(c),
                       np.cos(ang), np.sin(ang), w, ic, ir, K)
    np.testing.assert_allclose(F1, F2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(T1, T2, rtol=0, atol=1e-12)


@pytest.mark.parametrize("which", ["c4", "d2"])
def test_symmetrize(which):
    """SYMMETRIZE_FT: the oracle's restatement equals the reference's
    VOL_TRANSFORM_MAT_FT sums bit for bit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import symmetry_elements
    mats = dict(zip(("c4", "d2"), symmetry_elements()))[which]
    rng = np.random.default_rng(71)
    vdim = 20
    vol = (rng.standard_normal((vdim, vdim, vdim // 2 + 1))
           + 1j * rng.standard_normal((vdim, vdim, vdim // 2 + 1)))
    np.testing.assert_array_equal(O.symmetrize(vol, mats, 7.5), O.ref_symmetrize(vol, mats, 7.5))


@pytest.mark.parametrize("dim,N,gc,join,a,alpha", [
    (3, 16, True, False, 1.9, 15.0), (3, 16, True, True, 1.9, 10.0), (3, 12, False, False, 1.9, 15.0),
    (2, 48, True, False, 2.0, 15.0), (2, 32, False, True, 1.9, 15.0)])
def test_reconstruct(dim, N, gc, join, a, alpha):
    """oracle/reconstruct.py against Reconstructor::reconstruct of the compiled
    reference (src/Reconstructor.cpp:1129-1790, with the vendored FFTW and
    the build's trilinear correction) on fresh Hermitian-consistent inputs:
    the Wiener step, W balancing against the tabulated MKB kernel, 1/T, the
    inverse transform and the correction, to 1e-12 of the map's peak."""
    from oracle import reconstruct as RC
    rng = np.random.default_rng(100 * dim + N + int(gc) + 2 * int(join))
    pf = 2
    shape = (N * pf,) * dim
    F = np.fft.rfftn(rng.standard_normal(shape))
    T = np.abs(np.fft.rfftn(rng.standard_normal(shape))) ** 2 / np.prod(shape) + 0.5
    fsc = np.linspace(0.999, 0.1, N // 2 + 1)
    maxR = N // 2 - 1
    ref = O.ref_reconstruct(F, T, pf, maxR, fsc, join_half=join, grid_corr=gc, a=a, alpha=alpha)
    out, _ = RC.reconstruct(F, T, pf, maxR, fsc=fsc, join_half=join, grid_corr=gc, a=a, alpha=alpha)
    assert np.abs(out - ref).max() < 1e-12 * np.abs(ref).max()
