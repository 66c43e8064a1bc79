"""Write tests/golden/ref_golden.npz: inputs and outputs of the reference's
own compiled routines (oracle/_ref/libthunder_ref.so, built by
oracle/ref/Makefile from the THUNDER sources) on small seeded cases.

Also writes tests/golden/ref_golden_formats.npz (the 2-D, preprocessing,
transform, re-mask, spectrum and MRC routines) and tests/golden/ref_golden_recon.npz (the
symmetrisation of half transforms and the reconstruction chain).  Run in a checkout that has the THUNDER tree:
    python tests/golden/make_golden.py
The fixture pins the oracle (tests/test_oracle_golden.py) on machines that
do not have the reference sources."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "thunder-refactor-expectation_gb300"))

from oracle import oracle as O  # noqa: E402
from tg3 import synth  # noqa: E402


def main():
    R = O.ref()
    if R is None:
        raise SystemExit("reference cross-check library unavailable")
    rng = np.random.default_rng(20261203)
    g = {}
    box, pf = 16, 2
    iCol, iRow, iSig, iPxl = synth.pixel_index(box, 6, 1)
    K = len(iCol)
    g["iCol"], g["iRow"] = iCol, iRow
    g["box"], g["pf"] = box, pf

    # rotations
    q = synth.haar_quaternions(rng, 8)
    q[0] = (1, 0, 0, 0)
    mat = np.zeros((8, 9))
    R.ref_rotmat(q, 8, mat)
    g["rot_quat"], g["rot_mat"] = q, mat

    # projection: a blob map on the padded grid, rotations incl. identity
    bm = synth.blob_map(rng, 6, (2.0, 4.0), 1.5, 4.0)
    vol = np.ascontiguousarray(synth.padded_volume(bm, box, pf).numpy())
    proj = np.zeros((8, K), np.complex128)
    R.ref_project(vol, vol.shape[0], mat, 8, iCol, iRow, K, pf, proj)
    g["vol"], g["proj"] = vol, proj

    # phase shifts and an image shift
    t = np.array([[0.0, 0.0], [1.0, -2.0], [-2.5, 0.75], [3.0, 3.0]])
    tra = np.zeros((4, K), np.complex128)
    R.ref_translate(t, 4, box, iCol, iRow, K, tra)
    g["trans"], g["tra"] = t, tra

    # CTF
    attr = synth.ctf_attrs(rng, 3)
    ctf = np.zeros((3, K))
    for i in range(3):
        row = np.zeros(K)
        R.ref_ctf(np.ascontiguousarray(attr[i]), 1.5, box, iCol, iRow, K, row)
        ctf[i] = row
    g["ctf_attr"], g["ctf"] = attr, ctf

    # likelihood: image-major single and pixel-major batch
    dat = rng.standard_normal((4, K)) + 1j * rng.standard_normal((4, K))
    sig = -0.5 / (1 + rng.random((4, K)))
    cc = np.concatenate([ctf, ctf[:1]], 0)
    pri = proj[1] * tra[1]
    g["dvp_dat"], g["dvp_sig"], g["dvp_ctf"], g["dvp_pri"] = dat, sig, cc, pri
    g["dvp_one"] = np.array([R.ref_logdvp(np.ascontiguousarray(dat[0]), pri,
                                          np.ascontiguousarray(cc[0]),
                                          np.ascontiguousarray(sig[0]), K)])
    mn = np.zeros(4)
    R.ref_logdvp_mn(np.ascontiguousarray(dat.T), pri, np.ascontiguousarray(cc.T),
                    np.ascontiguousarray(sig.T), 4, K, mn)
    g["dvp_mn"] = mn

    # MKB table (a = 1.9, alpha = 15, b = (pf a)^2, n = 1e5): keep a sample
    tab = np.zeros(100001)
    R.ref_mkb_table(1.9, 15.0, (2 * 1.9) ** 2, 100000, tab)
    sel = np.unique(np.concatenate([np.arange(0, 25100, 97), [24999, 25000, 25001, 100000]]))
    g["mkb_idx"], g["mkb_val"] = sel, tab[sel]

    # insertion, both kernels, two slices each
    img = rng.standard_normal((2, K)) + 1j * rng.standard_normal((2, K))
    g["ins_img"], g["ins_w"] = img, np.array([0.3, 1.7])
    for kern in (0, 1):
        F = np.zeros(vol.shape, np.complex128)
        T = np.zeros(vol.shape)
        for s in range(2):
            R.ref_insert(F, T, vol.shape[0], np.ascontiguousarray(img[s]),
                         np.ascontiguousarray(ctf[s]), np.ascontiguousarray(mat[s + 1]),
                         float(g["ins_w"][s]), (iCol * pf).astype(np.int32),
                         (iRow * pf).astype(np.int32), K, kern, 1.9, 15.0,
                         (2 * 1.9) ** 2, 100000)
        nz = np.nonzero((np.abs(F) + np.abs(T)).ravel())[0]
        g[f"ins{kern}_idx"], g[f"ins{kern}_F"], g[f"ins{kern}_T"] = nz, F.ravel()[nz], T.ravel()[nz]

    # resampling: (n, nOut, narrowing)
    for c, (n, n_out, mode) in enumerate([(50, 40, 0), (100, 100, 1), (1000, 1000, 1)]):
        u = np.exp(3 * rng.standard_normal(n))
        if c == 1:
            u[rng.integers(0, n, 10)] = 0.0
        w = rng.random(n)
        w /= w.sum()
        perm = rng.permutation(n)
        u0 = rng.random() / n_out
        src = np.zeros(n_out, np.int32)
        wo = np.zeros(n_out)
        R.ref_resample(n, u, w, perm.astype(np.uint64), u0, n_out, mode, src, wo)
        g[f"rs{c}_u"], g[f"rs{c}_w"], g[f"rs{c}_perm"] = u, w, perm.astype(np.int32)
        g[f"rs{c}_u0"], g[f"rs{c}_mode"] = np.array([u0]), np.array([mode])
        g[f"rs{c}_src"], g[f"rs{c}_wout"] = src, wo

    # descending index sort with ties
    v = rng.integers(0, 6, 40).astype(np.float64)
    o = np.zeros(40, np.uint64)
    R.ref_sort_descend(v, 40, o)
    g["sort_v"], g["sort_idx"] = v, o.astype(np.int64)

    out = Path(__file__).resolve().parent / "ref_golden.npz"
    np.savez_compressed(out, **g)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


def symmetry_elements():
    """Non-identity elements of C4 about z and of D2 (rotations by 180 degrees
    about x, y and z): the symmetry sets of the pins."""
    def rz(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.0]])
    c4 = np.stack([rz(np.pi / 2 * k) for k in (1, 2, 3)])
    d2 = np.stack([np.diag([1.0, -1, -1]), np.diag([-1.0, 1, -1]), np.diag([-1.0, -1, 1])])
    return c4, d2


def main_recon():
    """ref_golden_recon.npz: the reference's symmetrisation of half
    transforms (SYMMETRIZE_FT through VOL_TRANSFORM_MAT_FT) and its
    reconstruction (Reconstructor::reconstruct, with the vendored FFTW)."""
    R = O.ref()
    if R is None:
        raise SystemExit("reference cross-check library unavailable")
    rng = np.random.default_rng(20261204)
    g = {}
    vdim = 16
    vol = (rng.standard_normal((vdim, vdim, vdim // 2 + 1))
           + 1j * rng.standard_normal((vdim, vdim, vdim // 2 + 1)))
    g["sym_vol"] = vol
    for name, mats in zip(("c4", "d2"), symmetry_elements()):
        g[f"sym_mats_{name}"] = mats
        g[f"sym_out_{name}"] = O.ref_symmetrize(vol, mats, 6.5)
    g["sym_r"] = 6.5
    # Reconstructor::reconstruct on Hermitian-consistent accumulators (F the
    # half transform of a real volume, T = |half transform|^2 + 0.5, real and
    # even), stored at float32 precision (exact as float64) to keep the file
    # small; 3-D with W balancing, with joinHalf and with W = 1/T on one pair
    # of accumulators, and 2-D with W balancing
    rng = np.random.default_rng(20261205)
    pf = 2
    for dim, N, flags in ((3, 12, ((True, False), (True, True), (False, False))),
                          (2, 32, ((True, False),))):
        shape = (N * pf,) * dim
        F = np.fft.rfftn(rng.standard_normal(shape)).astype(np.complex64)
        T = (np.abs(np.fft.rfftn(rng.standard_normal(shape))) ** 2 / np.prod(shape)
             + 0.5).astype(np.float32)
        fsc = np.linspace(0.999, 0.2, N // 2 + 2)
        maxR = N // 2
        g[f"reco{dim}_F"], g[f"reco{dim}_T"], g[f"reco{dim}_fsc"] = F, T, fsc
        g[f"reco{dim}_args"] = np.array([pf, maxR])
        g[f"reco{dim}_flags"] = np.array(flags, dtype=np.int32)
        g[f"reco{dim}_out"] = np.stack([
            O.ref_reconstruct(F, T, pf, maxR, fsc, join_half=join, grid_corr=gc)
            for gc, join in flags])
    out = ROOT / "tests" / "golden" / "ref_golden_recon.npz"
    np.savez_compressed(out, **g)
    print("wrote", out)


def main_formats():
    """ref_golden_formats.npz: the 2-D projection and insertion
    (Image::getByInterpolationFT, Image::addFT), image preprocessing
    (bgMeanStddev, bgStddev, softMask), powerSpectrum and the MRC reader."""
    import tempfile
    from tg3 import io
    R = O.ref()
    if R is None:
        raise SystemExit("reference cross-check library unavailable")
    rng = np.random.default_rng(20261204)
    g = {}
    box, pf = 16, 2
    vdim = box * pf
    iCol, iRow = synth.pixel_index(box, 6, 1)[:2]
    K = len(iCol)
    g["iCol"], g["iRow"], g["box"], g["pf"] = iCol, iRow, box, pf
    img = np.ascontiguousarray(rng.standard_normal((vdim, vdim // 2 + 1)) +
                               1j * rng.standard_normal((vdim, vdim // 2 + 1)))
    ang = rng.uniform(0, 2 * np.pi, 6)
    rot = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    p2 = np.zeros((6, K), np.complex128)
    R.ref_project2d(img, vdim, rot, 6, iCol, iRow, K, pf, p2)
    g["p2_img"], g["p2_rot"], g["p2"] = img, rot, p2
    F = np.zeros((vdim, vdim // 2 + 1), np.complex128)
    T = np.zeros((vdim, vdim // 2 + 1))
    ic, ir = np.ascontiguousarray(iCol * pf, np.int32), np.ascontiguousarray(iRow * pf, np.int32)
    ins_img = rng.standard_normal((3, K)) + 1j * rng.standard_normal((3, K))
    ins_ctf = rng.uniform(-1, 1, (3, K))
    ins_w = rng.uniform(0.2, 1.0, 3)
    for s in range(3):
        R.ref_insert2d(F, T, vdim, np.ascontiguousarray(ins_img[s]), np.ascontiguousarray(ins_ctf[s]),
                       rot[s, 0], rot[s, 1], float(ins_w[s]), ic, ir, K)
    g["i2_img"], g["i2_ctf"], g["i2_w"], g["i2_F"], g["i2_T"] = ins_img, ins_ctf, ins_w, F, T
    N, r = 32, 11.3
    c = np.arange(N) - N // 2
    xx, yy = np.meshgrid(c, c)
    imgs = 2.0 + 0.6 * rng.standard_normal((2, N, N)) + 3.0 * np.exp(-(xx ** 2 + yy ** 2) / 40.0)
    outs, stats = [], []
    for m in (1, 0):
        for l in range(2):
            o, st = np.zeros(N * N), np.zeros(3)
            R.ref_prep_image(np.ascontiguousarray(io.centred(imgs[l])).ravel(), N, r, m, o, st)
            outs.append(o.reshape(N, N))
            stats.append(st)
    g["pp_imgs"], g["pp_r"], g["pp_out"], g["pp_stats"] = imgs, np.array([r]), np.stack(outs), np.stack(stats)
    Fh = rng.standard_normal((N, N // 2 + 1)) + 1j * rng.standard_normal((N, N // 2 + 1))
    ps = np.zeros(15)
    R.ref_power_spectrum(np.ascontiguousarray(Fh), N, 15, ps)
    g["ps_F"], g["ps"] = Fh, ps
    stack = rng.standard_normal((2, 12, 12)).astype(np.float32)
    with tempfile.TemporaryDirectory() as td:
        path = str(Path(td) / "s.mrcs")
        io.write_mrc(path, stack)
        reads = []
        for s in range(2):
            o = np.zeros(144)
            if R.ref_read_mrc(path.encode(), s, 12, o):
                raise SystemExit("reference MRC read failed")
            reads.append(o.reshape(12, 12))
    g["mrc_stack"], g["mrc_ref"] = stack, np.stack(reads)
    # the preprocessing's transform (FFT::fw of an image held with its centre
    # at index 0) and the re-mask (reMaskImg: FFT::bw, soft mask, FFT::fw),
    # through the reference's FFT class on the vendored FFTW
    rng2 = np.random.default_rng(20261206)
    img = rng2.standard_normal((32, 32))
    g["fw_img"], g["fw_ref"] = img, O.ref_fw_image(img)
    Fm = np.fft.rfft2(rng2.standard_normal((32, 32)))
    g["remask_F"], g["remask_r"] = Fm, 9.5
    g["remask_ref"] = O.ref_remask(Fm, 9.5)
    out = Path(__file__).resolve().parent / "ref_golden_formats.npz"
    np.savez_compressed(out, **g)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
    main_formats()
    main_recon()
