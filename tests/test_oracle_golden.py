"""The oracle restatement against the reference's own outputs, stored in
tests/golden/ref_golden.npz by tests/golden/make_golden.py (which ran the
reference's compiled sources).  CPU only."""
import numpy as np
import pytest

from oracle import oracle as O


def test_rotmat(golden):
    m = O.rotmat(golden["rot_quat"]).reshape(-1, 9)
    assert np.array_equal(m, golden["rot_mat"])


def test_project_bit_exact(golden):
    m = golden["rot_mat"]
    P = O.project(golden["vol"], m, golden["iCol"], golden["iRow"], int(golden["pf"]))
    assert np.array_equal(P, golden["proj"])


def test_translate(golden):
    S = O.translate(golden["trans"], int(golden["box"]), golden["iCol"], golden["iRow"])
    np.testing.assert_allclose(S, golden["tra"], rtol=0, atol=1e-13)


def test_ctf(golden):
    c = O.ctf(golden["ctf_attr"], 1.5, int(golden["box"]), golden["iCol"], golden["iRow"])
    np.testing.assert_allclose(c, golden["ctf"], rtol=0, atol=1e-12)


def test_logdvp(golden):
    d, s, c, p = golden["dvp_dat"], golden["dvp_sig"], golden["dvp_ctf"], golden["dvp_pri"]
    assert O.logdvp(d[0], p, c[0], s[0]) == golden["dvp_one"][0]
    mn = np.array([O.logdvp(d[i], p, c[i], s[i]) for i in range(4)])
    np.testing.assert_allclose(mn, golden["dvp_mn"], rtol=1e-14)


def test_mkb_table(golden):
    tab = O.mkb_table(1.9, 15.0, (2 * 1.9) ** 2, 100000)
    idx = golden["mkb_idx"]
    np.testing.assert_allclose(tab[idx], golden["mkb_val"], rtol=1e-13, atol=1e-300)
    # support ends at r^2 = a^2 = 3.61 (index 25000 of 1e5 over 14.44)
    assert tab[25000] > 0 and tab[25001] == 0


def _insert(golden, kern):
    box, pf = int(golden["box"]), int(golden["pf"])
    vol = golden["vol"]
    F = np.zeros(vol.shape, np.complex128)
    T = np.zeros(vol.shape)
    tab = O.mkb_table(1.9, 15.0, (2 * 1.9) ** 2, 100000)
    for s in range(2):
        O.insert(F, T, golden["ins_img"][s], golden["ctf"][s],
                 golden["rot_mat"][s + 1], golden["ins_w"][s],
                 golden["iCol"] * pf, golden["iRow"] * pf, kern, 2 * 1.9, tab,
                 (2 * 1.9) ** 2)
    return F.ravel(), T.ravel()


def test_insert_trilinear_bit_exact(golden):
    F, T = _insert(golden, 0)
    idx = golden["ins0_idx"]
    assert np.count_nonzero(np.abs(F) + np.abs(T)) == len(idx)
    assert np.array_equal(F[idx], golden["ins0_F"])
    assert np.array_equal(T[idx], golden["ins0_T"])


def test_insert_mkb(golden):
    F, T = _insert(golden, 1)
    idx = golden["ins1_idx"]
    assert np.count_nonzero(np.abs(F) + np.abs(T)) == len(idx)
    np.testing.assert_allclose(F[idx], golden["ins1_F"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(T[idx], golden["ins1_T"], rtol=1e-12, atol=1e-14)


def test_resample_bit_exact(golden):
    for c in range(3):
        u, w, perm = golden[f"rs{c}_u"], golden[f"rs{c}_w"], golden[f"rs{c}_perm"]
        mode = int(golden[f"rs{c}_mode"][0])
        pfac = O.peak_factor_r(u) if mode else 0.0
        n_out = len(golden[f"rs{c}_src"])
        src, wout, _ = O.resample(u, w, perm, golden[f"rs{c}_u0"][0], pfac, n_out)
        assert np.array_equal(src, golden[f"rs{c}_src"]), c
        assert np.array_equal(wout, golden[f"rs{c}_wout"]), c


def test_descend_order_ties(golden):
    assert np.array_equal(O.descend_order(golden["sort_v"]), golden["sort_idx"])


def test_bessel_i0_series():
    scipy = __import__("pytest").importorskip("scipy.special")
    for x in (0.0, 0.5, 3.0, 7.5, 15.0):
        np.testing.assert_allclose(O.bessel_i0(x), scipy.i0(x), rtol=1e-14)


def test_project2d_golden(golden_formats):
    g = golden_formats
    P = O.project2d(g["p2_img"], g["p2_rot"], g["iCol"], g["iRow"], int(g["pf"]))
    np.testing.assert_allclose(P, g["p2"], rtol=0, atol=1e-12)


def test_insert2d_golden(golden_formats):
    g = golden_formats
    pf = int(g["pf"])
    F = np.zeros(g["i2_F"].shape, np.complex128)
    T = np.zeros(g["i2_T"].shape)
    ic = np.ascontiguousarray(g["iCol"] * pf, np.int32)
    ir = np.ascontiguousarray(g["iRow"] * pf, np.int32)
    for s in range(3):
        O.insert2d(F, T, g["i2_img"][s], g["i2_ctf"][s], g["p2_rot"][s], float(g["i2_w"][s]), ic, ir)
    np.testing.assert_allclose(F, g["i2_F"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(T, g["i2_T"], rtol=0, atol=1e-12)


def test_preprocess_golden(golden_formats):
    """Background normalisation, statistics and zero soft mask (masked, then
    unmasked) against the reference's bgMeanStddev / bgStddev / softMask."""
    from oracle import preprocess as PP
    g = golden_formats
    r = float(g["pp_r"][0])
    k = 0
    for mask in (True, False):
        for img in g["pp_imgs"]:
            y, st = PP.normalise(img, r)
            y = PP.soft_mask(y, r) if mask else y
            np.testing.assert_allclose(np.fft.ifftshift(y), g["pp_out"][k], rtol=0, atol=1e-12)
            np.testing.assert_allclose(st, g["pp_stats"][k], rtol=1e-13)
            k += 1


def test_power_spectrum_golden(golden_formats):
    from oracle import preprocess as PP
    g = golden_formats
    np.testing.assert_allclose(PP.power_spectrum(g["ps_F"], len(g["ps"])), g["ps"], rtol=1e-13)


def test_mrc_reader_golden(golden_formats, tmp_path):
    """The library's MRC writer and reader against the reference's
    ImageFile read of the same stack (its in-memory layout is the centred
    reindexing of the file order)."""
    from tg3 import io
    g = golden_formats
    p = tmp_path / "s.mrcs"
    io.write_mrc(p, g["mrc_stack"])
    got = io.read_mrc(p)
    for s in range(len(got)):
        np.testing.assert_array_equal(io.centred(got[s]), g["mrc_ref"][s])


@pytest.mark.parametrize("which", ["c4", "d2"])
def test_symmetrize_matches_reference_fixture(which):
    """The oracle's SYMMETRIZE_FT against the reference's output recorded in
    tests/golden/ref_golden_recon.npz (tests/golden/make_golden.py)."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_golden_recon.npz")
    out = O.symmetrize(g["sym_vol"], g[f"sym_mats_{which}"], float(g["sym_r"]))
    np.testing.assert_array_equal(out, g[f"sym_out_{which}"])


@pytest.mark.parametrize("dim", [3, 2])
def test_reconstruct_matches_reference_fixture(dim):
    """oracle/reconstruct.py against the reference's Reconstructor::reconstruct
    (compiled with the vendored FFTW) recorded in tests/golden/ref_golden_recon.npz:
    W balancing (with and without joinHalf) and W = 1/T in 3-D, balancing in 2-D."""
    from pathlib import Path
    from oracle import reconstruct as RC
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_golden_recon.npz")
    pf, maxR = (int(v) for v in g[f"reco{dim}_args"])
    for (gc, join), ref in zip(g[f"reco{dim}_flags"], g[f"reco{dim}_out"]):
        out, _ = RC.reconstruct(g[f"reco{dim}_F"], g[f"reco{dim}_T"], pf, maxR,
                                fsc=g[f"reco{dim}_fsc"], join_half=bool(join), grid_corr=bool(gc))
        assert np.abs(out - ref).max() < 1e-12 * np.abs(ref).max()


def test_transform_and_remask_match_reference_fixture():
    """The preprocessing's transform (numpy's rfft2 of the image held with its
    centre at index 0) and oracle/preprocess.py remask against the reference's
    FFT::fw and reMaskImg on the vendored FFTW, recorded in
    tests/golden/ref_golden_formats.npz."""
    from pathlib import Path
    from oracle import preprocess as PP
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref_golden_formats.npz")
    F = np.fft.rfft2(g["fw_img"])
    assert np.abs(F - g["fw_ref"]).max() < 1e-12 * np.abs(g["fw_ref"]).max()
    got = PP.remask(g["remask_F"][None], float(g["remask_r"]))[0]
    assert np.abs(got - g["remask_ref"]).max() < 1e-12 * np.abs(g["remask_ref"]).max()
