"""Reconstruction on the GPU (tg3_ctx_reconstruct_d) against the oracle's
restatement of Reconstructor::reconstruct (oracle/reconstruct.py): Wiener
filter from the FSC, W by balancing against the MKB kernel or 1 / T, the
inverse transform of F W, the central N^3 and the gridding correction.  F
and T are Hermitian-consistent (F the transform of a real map, T radial), as
sums over whole slices are in the limit: an inverse real transform of a
half grid is otherwise implementation-defined."""
import numpy as np
import pytest
import torch

import tg3
from oracle import oracle as O
from oracle import reconstruct as RC

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _inputs(rng, N, pf):
    vdim = N * pf
    c = np.arange(vdim) - vdim // 2
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    m = np.zeros((vdim, vdim, vdim))
    for _ in range(8):
        p = rng.uniform(-N / 5, N / 5, 3)
        m += np.exp(-((x - p[0]) ** 2 + (y - p[1]) ** 2 + (z - p[2]) ** 2) / (2 * rng.uniform(1.5, 3) ** 2))
    q = np.fft.fftfreq(vdim, 1.0 / vdim)
    kz, ky, kx = np.meshgrid(q, q, np.arange(vdim // 2 + 1), indexing="ij")
    k = np.sqrt(kx * kx + ky * ky + kz * kz)
    T = 50.0 * np.exp(-k / (0.4 * vdim)) + 0.5
    F = np.fft.rfftn(np.fft.ifftshift(m)) * T / 40.0
    return F, T


@pytest.mark.parametrize("grid_corr,kernel", [(True, tg3.KERNEL_TRILINEAR), (False, tg3.KERNEL_MKB),
                                              (True, tg3.KERNEL_MKB)])
def test_reconstruct_matches_oracle(grid_corr, kernel):
    rng = np.random.default_rng(7 + kernel)
    N, pf, maxR = 32, 2, 14
    F, T = _inputs(rng, N, pf)
    fsc = np.clip(1.05 - np.arange(N // 2 + 1) / (N / 2), 0, 1)
    ctx = tg3.Context(0)
    try:
        ctx.insert_begin(N * pf, pf)
        ctx.insert_load(torch.as_tensor(F.astype(np.complex64)).to(DEV),
                        torch.as_tensor(T.astype(np.float32)).to(DEV))
        vol = torch.empty((N, N, N), dtype=torch.float32, device=DEV)
        rounds = ctx.reconstruct(vol, maxR, fsc=torch.as_tensor(fsc).to(DEV), join_half=True,
                                 grid_corr=grid_corr, kernel=kernel)
        ctx.sync()
    finally:
        ctx.close()
    ref, ref_rounds = RC.reconstruct(F, T, pf, maxR, fsc=fsc, join_half=True, grid_corr=grid_corr,
                                     kernel="mkb" if kernel == tg3.KERNEL_MKB else "trilinear")
    got = vol.cpu().numpy()
    assert rounds == ref_rounds
    assert np.abs(got - ref).max() < 1e-3 * np.abs(ref).max()


def _inputs2d(rng, N, pf):
    vdim = N * pf
    c = np.arange(vdim) - vdim // 2
    y, x = np.meshgrid(c, c, indexing="ij")
    m = np.zeros((vdim, vdim))
    for _ in range(6):
        p = rng.uniform(-N / 5, N / 5, 2)
        m += np.exp(-((x - p[0]) ** 2 + (y - p[1]) ** 2) / (2 * rng.uniform(1.5, 3) ** 2))
    q = np.fft.fftfreq(vdim, 1.0 / vdim)
    ky, kx = np.meshgrid(q, np.arange(vdim // 2 + 1), indexing="ij")
    k = np.sqrt(kx * kx + ky * ky)
    T = 50.0 * np.exp(-k / (0.4 * vdim)) + 0.5
    F = np.fft.rfft2(np.fft.ifftshift(m)) * T / 40.0
    return F, T


@pytest.mark.parametrize("grid_corr,kernel", [(True, tg3.KERNEL_TRILINEAR), (False, tg3.KERNEL_MKB),
                                              (True, tg3.KERNEL_MKB)])
def test_reconstruct_2d_matches_oracle(grid_corr, kernel):
    """tg3_Reconstruct2D (MODE_2D: the 2-D accumulators of one class, host
    buffers) against the oracle's 2-D chain: the same number of balancing
    rounds and the image within 1e-3 of its peak."""
    rng = np.random.default_rng(17 + kernel)
    N, pf, maxR = 64, 2, 28
    F, T = _inputs2d(rng, N, pf)
    fsc = np.clip(1.05 - np.arange(N // 2 + 1) / (N / 2), 0, 1)
    img = np.zeros((N, N), np.float32)
    rounds = np.zeros(1, np.int32)
    # named arrays: the addresses passed must stay alive through the call
    F32 = np.ascontiguousarray(F.astype(np.complex64))
    T32 = np.ascontiguousarray(T.astype(np.float32))
    tg3.check(tg3.lib().tg3_Reconstruct2D(tg3.ptr(F32), tg3.ptr(T32), N * pf, pf, tg3.ptr(fsc),
                                          len(fsc), 1, maxR, int(grid_corr), kernel, 1.9, 15.0,
                                          tg3.ptr(img), tg3.ptr(rounds)))
    ref, ref_rounds = RC.reconstruct(F, T, pf, maxR, fsc=fsc, join_half=True, grid_corr=grid_corr,
                                     kernel="mkb" if kernel == tg3.KERNEL_MKB else "trilinear")
    assert int(rounds[0]) == ref_rounds
    assert np.abs(img - ref).max() < 1e-3 * np.abs(ref).max()


def _golden_recon():
    from pathlib import Path
    return np.load(Path(__file__).resolve().parent / "golden" / "ref_golden_recon.npz")


@pytest.mark.parametrize("case", [0, 1, 2])
def test_reconstruct_matches_reference_fixture(case):
    """tg3_ctx_reconstruct_d against the reference's own
    Reconstructor::reconstruct (compiled with the vendored FFTW; outputs in
    tests/golden/ref_golden_recon.npz): W balancing, joinHalf, W = 1/T; the
    build's trilinear correction.  The map within 1e-3 of its peak, with the
    balancing rounds of the oracle (which matches the fixture to 1e-14)."""
    g = _golden_recon()
    pf, maxR = (int(v) for v in g["reco3_args"])
    gc, join = (bool(v) for v in g["reco3_flags"][case])
    F, T, fsc = g["reco3_F"], g["reco3_T"], g["reco3_fsc"]
    N = F.shape[0] // pf
    ctx = tg3.Context(0)
    try:
        ctx.insert_begin(N * pf, pf)
        ctx.insert_load(torch.as_tensor(F).to(DEV), torch.as_tensor(T).to(DEV))
        vol = torch.empty((N, N, N), dtype=torch.float32, device=DEV)
        rounds = ctx.reconstruct(vol, maxR, fsc=torch.as_tensor(fsc).to(DEV), join_half=join,
                                 grid_corr=gc, kernel=tg3.KERNEL_TRILINEAR)
        ctx.sync()
    finally:
        ctx.close()
    ref = g["reco3_out"][case]
    _, ref_rounds = RC.reconstruct(F, T, pf, maxR, fsc=fsc, join_half=join, grid_corr=gc)
    assert rounds == ref_rounds
    assert np.abs(vol.cpu().numpy() - ref).max() < 1e-3 * np.abs(ref).max()


def test_reconstruct_2d_matches_reference_fixture():
    """tg3_Reconstruct2D against the reference's MODE_2D reconstruct
    (tests/golden/ref_golden_recon.npz), W balancing, trilinear correction."""
    g = _golden_recon()
    pf, maxR = (int(v) for v in g["reco2_args"])
    gc, join = (bool(v) for v in g["reco2_flags"][0])
    F = np.ascontiguousarray(g["reco2_F"])
    T = np.ascontiguousarray(g["reco2_T"])
    fsc = np.ascontiguousarray(g["reco2_fsc"])
    N = F.shape[0] // pf
    img = np.zeros((N, N), np.float32)
    rounds = np.zeros(1, np.int32)
    tg3.check(tg3.lib().tg3_Reconstruct2D(tg3.ptr(F), tg3.ptr(T), N * pf, pf, tg3.ptr(fsc),
                                          len(fsc), int(join), maxR, int(gc),
                                          tg3.KERNEL_TRILINEAR, 1.9, 15.0, tg3.ptr(img),
                                          tg3.ptr(rounds)))
    ref = g["reco2_out"][0]
    _, ref_rounds = RC.reconstruct(F, T, pf, maxR, fsc=fsc, join_half=join, grid_corr=gc)
    assert int(rounds[0]) == ref_rounds
    assert np.abs(img - ref).max() < 1e-3 * np.abs(ref).max()


@pytest.mark.parametrize("which", ["c4", "d2"])
def test_prepare_tf_matches_oracle(which):
    """PrepareTF on the accumulators: F and T scaled by 1 / T at the origin,
    then symmetrised over the elements of C4 or D2 within maxRadius pf + 1,
    T floored -- against the oracle's SYMMETRIZE_FT (pinned bit for bit to
    the reference's), within 1e-5 of the peak; and the reference-shaped host
    form against the device form."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import symmetry_elements
    mats = dict(zip(("c4", "d2"), symmetry_elements()))[which]
    rng = np.random.default_rng(83)
    box, pf, maxR = 24, 2, 10
    vd = box * pf
    shape = (vd, vd, vd // 2 + 1)
    F = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    T = (rng.random(shape) + 0.5).astype(np.float32)
    ctx = tg3.Context(0)
    try:
        ctx.insert_begin(vd, pf)
        ctx.insert_load(torch.as_tensor(F).to(DEV), torch.as_tensor(T).to(DEV))
        ctx.prepare_tf(mats, maxR)
        Fo = torch.empty(shape + (2,), dtype=torch.float32, device=DEV)
        To = torch.empty(shape, dtype=torch.float32, device=DEV)
        ctx.insert_read(Fo, To)
        ctx.sync()
        Fg = Fo.cpu().numpy().view(np.complex64)[..., 0]
        Tg = To.cpu().numpy()
    finally:
        ctx.close()
    sf = 1.0 / float(T[0, 0, 0])
    r = maxR * pf + 1.0
    Fr = O.symmetrize(F.astype(np.complex128) * sf, mats, r)
    Tr = np.maximum(O.symmetrize(T.astype(np.float64) * sf, mats, r).real, 1e-25)
    assert np.abs(Fg - Fr).max() < 1e-5 * np.abs(Fr).max()
    assert np.abs(Tg - Tr).max() < 1e-5 * np.abs(Tr).max()
    Fh, Th = F.copy(), T.copy()
    tg3.check(tg3.lib().tg3_PrepareTF(tg3.ptr(Fh), tg3.ptr(Th), vd,
                                      tg3.ptr(np.ascontiguousarray(mats.reshape(-1, 9))),
                                      len(mats), maxR, pf))
    np.testing.assert_array_equal(Fh, Fg)
    np.testing.assert_array_equal(Th, Tg)
