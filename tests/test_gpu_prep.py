"""Image preprocessing on the GPU (tg3_prepare_images_d) against the oracle's
restatement of the reference's chain (oracle/preprocess.py, pinned to the
compiled reference on the CPU): background normalisation, zero soft mask,
1 / stdN, transform of the centred image, pixel gather.  Inputs are read
from an MRC stack written and read by the library."""
import numpy as np
import pytest
import torch

import tg3
from oracle import preprocess as PP
from tg3 import io, synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _stack(rng, n, N):
    c = np.arange(N) - N // 2
    i, j = np.meshgrid(c, c)
    out = []
    for _ in range(n):
        img = 2.0 + 0.5 * rng.standard_normal((N, N))
        for _ in range(6):
            x0, y0 = rng.uniform(-N / 6, N / 6, 2)
            img += rng.uniform(1, 3) * np.exp(-((i - x0) ** 2 + (j - y0) ** 2) /
                                              (2 * rng.uniform(2, 4) ** 2))
        out.append(img)
    return np.stack(out).astype(np.float32)


@pytest.mark.parametrize("mask,std_n", [(1, 0.0), (0, 0.0), (1, 1.3)])
def test_prepare_images_matches_oracle(tmp_path, mask, std_n):
    rng = np.random.default_rng(40 + mask)
    N, n, r = 64, 37, 24.5
    io.write_mrc(tmp_path / "p.mrcs", _stack(rng, n, N), pixel_size=1.5)
    imgs = io.read_mrc(tmp_path / "p.mrcs")
    iCol, iRow = synth.pixel_index(N, 20, synth.config_rL(N, 1.5))[:2]
    K = len(iCol)
    ctx = tg3.Context(0)
    try:
        ctx.set_pixels(iCol, iRow, N)
        dat = torch.empty((n, K), dtype=torch.complex64, device=DEV)
        stats = torch.empty((n, 3), dtype=torch.float32, device=DEV)
        ctx.prepare_images(torch.as_tensor(imgs).to(DEV), r, dat, mask=bool(mask), std_n=std_n,
                           stats=stats)
        ctx.sync()
    finally:
        ctx.close()
    ref, st, _ = PP.preprocess(imgs, r, iCol, iRow, mask=bool(mask), std_n=std_n or None)
    got = dat.cpu().numpy()
    assert np.abs(got - ref).max() < 2e-5 * np.abs(ref).max()
    np.testing.assert_allclose(stats.cpu().numpy(), st, rtol=2e-6)


def test_prepare_images_rejects_mismatched_pixel_set():
    ctx = tg3.Context(0)
    try:
        iCol, iRow = synth.pixel_index(32, 10, 1)[:2]
        ctx.set_pixels(iCol, iRow, 32)
        img = torch.zeros((2, 64, 64), dtype=torch.float32, device=DEV)
        dat = torch.empty((2, len(iCol)), dtype=torch.complex64, device=DEV)
        with pytest.raises(tg3.TG3Error):
            ctx.prepare_images(img, 20.0, dat)
    finally:
        ctx.close()


@pytest.mark.parametrize("by_group", [True, False])
def test_sigma_matches_oracle(by_group):
    """Noise spectrum from the images at their best poses (allReduceSigma)
    against the oracle's restatement over the same pixel data."""
    from oracle import oracle as O
    rng = np.random.default_rng(50 + by_group)
    N, pf, px, r = 32, 2, 1.5, 15
    bm = synth.blob_map(rng, 16, (2.0, 4.0), px, 8.0)
    vol = synth.padded_volume(bm, N, pf).numpy().astype(np.complex64)
    iCol, iRow = io.spectrum_pixels(N, r)
    K = len(iCol)
    n, n_group = 40, 3
    quats = synth.haar_quaternions(rng, n)
    mats = synth.quat_to_mat(quats).reshape(n, 9)
    trans = rng.uniform(-2, 2, (n, 2))
    offset = rng.uniform(-0.5, 0.5, (n, 2))
    groups = rng.integers(1, n_group + 1, n).astype(np.int32)
    ctf = synth.ctf_values(synth.ctf_attrs(rng, n), px, N, iCol, iRow).astype(np.float32)
    P = O.project(vol.astype(np.complex128), mats, iCol, iRow, pf)
    models = np.stack([ctf[l] * P[l] * synth.phase_shift(trans[l], N, iCol, iRow)[0]
                       for l in range(n)])
    noise = lambda: 0.4 * (rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K)))
    datM = (models + noise()).astype(np.complex64)
    datN = (models * np.exp(2j * np.pi * (np.outer(offset[:, 0], iCol) + np.outer(offset[:, 1], iRow)) / N)
            + noise()).astype(np.complex64)
    d = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(DEV)
    sig = torch.empty((n_group, r), dtype=torch.float64, device=DEV)
    rcp = torch.empty_like(sig)
    ctx = tg3.Context(0)
    try:
        ctx.set_volume(0, d(vol), pf)
        ctx.set_pixels(iCol, iRow, N)
        ctx.sigma(0, d(datM), d(datN), d(ctf), d(mats), d(trans), d(offset), d(groups), n_group, r,
                  60.0, px, sig, rcp, by_group=by_group)
        ctx.sync()
    finally:
        ctx.close()
    rs, rr = PP.sigma(models, datM.astype(np.complex128), datN.astype(np.complex128), offset, iCol,
                      iRow, N, r, groups, n_group, by_group, 60.0, px)
    np.testing.assert_allclose(sig.cpu().numpy(), rs, rtol=2e-4)
    np.testing.assert_allclose(rcp.cpu().numpy(), rr, rtol=2e-4)


def test_remask_matches_oracle():
    """Re-masking of image transforms (the reference's reMask / reMaskImg):
    device form and the reference-shaped host form (in place, one host array
    per image) against the oracle's restatement (normalised inverse
    transform, soft mask about the centre, forward transform), within 2e-5
    of the largest value."""
    rng = np.random.default_rng(47)
    N, n, r, px = 64, 9, 22.0, 1.5
    real = np.fft.ifftshift(_stack(rng, n, N).astype(np.float64), axes=(-2, -1))
    F = np.fft.rfft2(real).astype(np.complex64)          # Hermitian-consistent, centre at 0
    ref = PP.remask(F.astype(np.complex128), r / px, 6.0)
    ctx = tg3.Context(0)
    try:
        out = ctx.remask(torch.as_tensor(F).to(DEV), r / px)
        ctx.sync()
        got = out.cpu().numpy()
    finally:
        ctx.close()
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() < 2e-5 * scale
    imgs = [np.ascontiguousarray(F[l]) for l in range(n)]
    ptrs = (np.ctypeslib.ctypes.c_void_p * n)(*[a.ctypes.data for a in imgs])
    tg3.check(tg3.lib().tg3_ReMask(ptrs, n, N, r, px, 6.0))
    assert np.abs(np.stack(imgs) - ref).max() < 2e-5 * scale
