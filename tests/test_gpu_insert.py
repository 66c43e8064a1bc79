"""MKB insertion's two GPU forms: the scatter (each pixel's support voxels,
one atomic each, the order of Reconstructor::insertP,
src/Reconstructor.cpp:782-863; the default) and the gather (each voxel of a
slice's slab summed from its pixels, one atomic; TG3_OPT_INSERT_GATHER).

- A pixel list that holds a pixel twice takes the scatter form even with
  the gather asked for, and still matches the double-precision oracle.
- At the production size (box 256, pf 2, cutoff 80, K = 9,930) both forms
  match the oracle (relative L2 1e-4, FSC >= 0.999 to the cutoff shell) and
  their bookkeeping (offset sum, counter) is identical."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _f32(x):
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.astype(np.complex64).astype(np.complex128)
    return x.astype(np.float32).astype(np.float64)


def _run(box, pf, iCol, iRow, dat, ctf, q, t, off, w, gather):
    vdim = pf * box
    c = tg3.Context(0)
    try:
        c.set_pixels(iCol, iRow, box)
        c.set_option(tg3.OPT_INSERT_GATHER, gather)
        c.insert_begin(vdim, pf)
        O3D = torch.zeros(3, dtype=torch.float64, device=DEV)
        cnt = torch.zeros(1, dtype=torch.int32, device=DEV)
        d = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(DEV)
        c.insert(len(q), d(dat), d(ctf), d(q), d(t), d(off), d(w), tg3.KERNEL_MKB, O3D, cnt)
        F = torch.empty((vdim, vdim, vdim // 2 + 1, 2), dtype=torch.float32, device=DEV)
        T = torch.empty((vdim, vdim, vdim // 2 + 1), dtype=torch.float32, device=DEV)
        c.insert_read(F, T)
        c.sync()
        return F, T, O3D.cpu().numpy(), int(cnt.item())
    finally:
        c.close()


def test_duplicate_pixel_takes_the_scatter_form():
    rng = np.random.default_rng(41)
    box, pf, px = 24, 2, 1.5
    iCol, iRow = synth.pixel_index(box, 9, synth.config_rL(box, px))[:2]
    iCol = np.concatenate([iCol, iCol[5:6]]).astype(np.int32)
    iRow = np.concatenate([iRow, iRow[5:6]]).astype(np.int32)
    K, nP = len(iCol), 5
    q = synth.haar_quaternions(rng, nP)
    t = np.zeros((nP, 2))
    w = rng.uniform(0.5, 1.5, nP).astype(np.float32)
    dat = (rng.standard_normal((nP, K)) + 1j * rng.standard_normal((nP, K))).astype(np.complex64)
    ctf = rng.uniform(-1, 1, (nP, K)).astype(np.float32)
    F, T, _, cnt = _run(box, pf, iCol, iRow, dat, ctf, q, t, np.zeros((nP, 2)), w, 1)
    assert cnt == nP
    vdim = pf * box
    Fg = F.cpu().numpy().astype(np.float64)
    Fg = Fg[..., 0] + 1j * Fg[..., 1]
    Fr = np.zeros((vdim, vdim, vdim // 2 + 1), np.complex128)
    Tr = np.zeros(Fr.shape)
    b = (pf * 1.9) ** 2
    tab = O.mkb_table(1.9, 15.0, b, 100000)
    mats = O.rotmat(q)
    for l in range(nP):
        O.insert(Fr, Tr, _f32(dat[l]), _f32(ctf[l]), mats[l], float(w[l]), iCol * pf, iRow * pf,
                 tg3.KERNEL_MKB, pf * 1.9, tab, b)
    assert np.abs(Fg - Fr).max() < 2e-4 * np.abs(Fr).max()
    assert np.abs(T.cpu().numpy() - Tr).max() < 2e-4 * Tr.max()


def test_both_forms_match_the_oracle_at_box_256():
    rng = np.random.default_rng(43)
    box, pf, px, rU = 256, 2, 1.1, 80
    iCol, iRow = synth.pixel_index(box, rU, synth.config_rL(box, px))[:2]
    K, nP = len(iCol), 12
    assert K == 9930
    q = synth.haar_quaternions(rng, nP)
    t = rng.uniform(-8, 8, (nP, 2))
    off = rng.uniform(-1, 1, (nP, 2))
    w = rng.uniform(0.5, 1.5, nP).astype(np.float32)
    dat = (rng.standard_normal((nP, K)) + 1j * rng.standard_normal((nP, K))).astype(np.complex64)
    ctf = rng.uniform(-1, 1, (nP, K)).astype(np.float32)
    Fa, Ta, Oa, ca = _run(box, pf, iCol, iRow, dat, ctf, q, t, off, w, 1)
    Fb, Tb, Ob, cb = _run(box, pf, iCol, iRow, dat, ctf, q, t, off, w, 0)
    assert ca == cb == nP
    np.testing.assert_allclose(Oa, Ob, rtol=1e-12, atol=1e-9)
    vdim = pf * box
    Fr = np.zeros((vdim, vdim, vdim // 2 + 1), np.complex128)
    Tr = np.zeros(Fr.shape)
    b = (pf * 1.9) ** 2
    tab = O.mkb_table(1.9, 15.0, b, 100000)
    mats = O.rotmat(q)
    for l in range(nP):
        tt = _f32(t[l]) - _f32(off[l])
        img = O.translate_image(_f32(dat[l]), -tt[0], -tt[1], box, iCol, iRow)
        O.insert(Fr, Tr, img, _f32(ctf[l]), mats[l], float(w[l]), iCol * pf, iRow * pf,
                 tg3.KERNEL_MKB, pf * 1.9, tab, b)
    fs, ts = np.abs(Fr).max(), Tr.max()
    nzr = int((Tr != 0).sum())
    # FP32 coordinates at radius ~160 move the table index rint(r^2 n / b) by
    # one step at some voxels; one step changes the MKB weight by ~3e-4 of
    # itself.  Measured on GB300: max 2.2-2.9e-4 of the peak, relative L2
    # 3.6-3.8e-5, FSC 1 - 2e-9, for both forms.
    for F, T in ((Fa, Ta), (Fb, Tb)):
        Fg = F.cpu().numpy().astype(np.float64)
        Fg = Fg[..., 0] + 1j * Fg[..., 1]
        Tg = T.cpu().numpy()
        assert np.abs(Fg - Fr).max() < 1e-3 * fs
        assert np.abs(Tg - Tr).max() < 1e-3 * ts
        assert np.linalg.norm(Fg - Fr) < 1e-4 * np.linalg.norm(Fr)
        assert np.linalg.norm(Tg - Tr) < 1e-4 * np.linalg.norm(Tr)
        f = O.fsc(Fg, Fr, int(rU * pf))
        assert f[1:].min() >= 0.999, f
        assert abs(int((Tg != 0).sum()) - nzr) <= 1e-5 * nzr
        del Fg, Tg


def test_fsc_matches_the_oracle():
    rng = np.random.default_rng(47)
    vdim, n_shell = 48, 24
    shape = (vdim, vdim, vdim // 2 + 1)
    A = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    B = (A + 0.7 * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))).astype(
        np.complex64)
    B[..., 3] = 0                 # shells with data in one volume only
    got = tg3.fsc(torch.as_tensor(A).to(DEV), torch.as_tensor(B).to(DEV), n_shell).cpu().numpy()
    ref = O.fsc(A.astype(np.complex128), B.astype(np.complex128), n_shell)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14)
    # identical volumes correlate fully in every shell that holds data
    one = tg3.fsc(torch.as_tensor(A).to(DEV), torch.as_tensor(A).to(DEV), n_shell).cpu().numpy()
    np.testing.assert_allclose(one, 1.0, rtol=0, atol=1e-12)


def test_insert_ratio_is_F_over_T():
    rng = np.random.default_rng(53)
    box, pf, px = 24, 2, 1.5
    iCol, iRow = synth.pixel_index(box, 9, synth.config_rL(box, px))[:2]
    K, nP = len(iCol), 7
    vdim = pf * box
    d = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(DEV)
    q = synth.haar_quaternions(rng, nP)
    dat = (rng.standard_normal((nP, K)) + 1j * rng.standard_normal((nP, K))).astype(np.complex64)
    ctf = rng.uniform(-1, 1, (nP, K)).astype(np.float32)
    c = tg3.Context(0)
    try:
        c.set_pixels(iCol, iRow, box)
        c.insert_begin(vdim, pf)
        c.insert(nP, d(dat), d(ctf), d(q), d(np.zeros((nP, 2))), None,
                 d(np.ones(nP, np.float32)), tg3.KERNEL_MKB)
        F = torch.empty((vdim, vdim, vdim // 2 + 1, 2), dtype=torch.float32, device=DEV)
        T = torch.empty((vdim, vdim, vdim // 2 + 1), dtype=torch.float32, device=DEV)
        V = torch.empty((vdim, vdim, vdim // 2 + 1), dtype=torch.complex64, device=DEV)
        c.insert_read(F, T)
        floor = 1e-3 * float(T.max())
        c.insert_ratio(V, floor)
        c.sync()
    finally:
        c.close()
    F, T, V = F.cpu().numpy(), T.cpu().numpy(), V.cpu().numpy()
    keep = T > floor
    ref = np.where(keep, (F[..., 0] + 1j * F[..., 1]) / np.where(keep, T, 1.0), 0)
    np.testing.assert_allclose(V, ref.astype(np.complex64), rtol=1e-6, atol=0)
    assert keep.sum() > 1000 and np.all(V[~keep] == 0)
