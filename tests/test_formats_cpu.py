"""Input formats and preprocessing on the CPU.
- The library's MRC reader against the reference's compiled ImageFile.
- The oracle's preprocessing against the reference's compiled bgMeanStddev,
  bgStddev and softMask, and with the transform and the re-mask through the
  reference's FFT class on the vendored FFTW.
- .thu databases: saveDatabase-formatted lines, round trips and malformed
  input."""
import numpy as np
import pytest

import tg3
from oracle import oracle as O
from oracle import preprocess as PP
from tg3 import io

R = O.ref()
needs_ref = pytest.mark.skipif(R is None, reason="reference cross-check library not built")


def _images(rng, n, N):
    """Smooth blobs on a noisy background with an offset, file order."""
    c = np.arange(N) - N // 2
    i, j = np.meshgrid(c, c)
    out = []
    for _ in range(n):
        img = 3.0 + 0.7 * rng.standard_normal((N, N))
        for _ in range(5):
            x0, y0 = rng.uniform(-N / 6, N / 6, 2)
            img += rng.uniform(1, 4) * np.exp(-((i - x0) ** 2 + (j - y0) ** 2) / (2 * rng.uniform(2, 5) ** 2))
        out.append(img)
    return np.stack(out)


@needs_ref
def test_mrc_read_matches_reference_imagefile(tmp_path):
    rng = np.random.default_rng(3)
    N = 32
    stack = rng.standard_normal((3, N, N)).astype(np.float32)
    p = tmp_path / "s.mrcs"
    io.write_mrc(p, stack, pixel_size=1.25)
    nx, ny, nz, mode, px = io.mrc_info(p)
    assert (nx, ny, nz, mode) == (N, N, 3) + (2,) and abs(px - 1.25) < 1e-6
    got = io.read_mrc(p)
    np.testing.assert_array_equal(got, stack)
    for s in range(3):
        ref = np.zeros(N * N)
        assert R.ref_read_mrc(str(p).encode(), s, N, ref) == 0
        np.testing.assert_array_equal(io.centred(got[s]).ravel(), ref)


@pytest.mark.parametrize("mode,dtype", [(0, np.int8), (1, np.int16), (6, np.uint16)])
def test_mrc_integer_modes(tmp_path, mode, dtype):
    """Integer stacks (a hand-made header with an extended header) read as
    float32 values."""
    rng = np.random.default_rng(mode)
    nx, ny, nz, ext = 6, 5, 4, 80
    info = np.iinfo(dtype)
    data = rng.integers(info.min, info.max, (nz, ny, nx), endpoint=True).astype(dtype)
    head = np.zeros(256, np.int32)
    head[:4] = (nx, ny, nz, mode)
    head[23] = ext                      # nsymbt, byte 92
    p = tmp_path / "i.mrc"
    p.write_bytes(head.tobytes() + b"\x01" * ext + data.tobytes())
    np.testing.assert_array_equal(io.read_mrc(p, 1, 2), data[1:3].astype(np.float32))


def test_mrc_errors(tmp_path):
    p = tmp_path / "bad.mrc"
    p.write_bytes(b"\x00" * 100)
    with pytest.raises(tg3.TG3Error):
        io.mrc_info(p)
    q = tmp_path / "s.mrc"
    io.write_mrc(q, np.zeros((2, 4, 4), np.float32))
    with pytest.raises(tg3.TG3Error):
        io.read_mrc(q, 1, 2)
    head = np.zeros(256, np.int32)
    head[:4] = (4, 4, 1, 4)             # complex mode: not an image stack
    r = tmp_path / "c.mrc"
    r.write_bytes(head.tobytes() + b"\x00" * 128)
    with pytest.raises(tg3.TG3Error):
        io.read_mrc(r)


@needs_ref
@pytest.mark.parametrize("mask", [1, 0])
def test_preprocessing_oracle_matches_reference(mask):
    """Background normalisation, its statistics and the zero soft mask of the
    oracle against the reference's bgMeanStddev / bgStddev / softMask on the
    same image, in the reference's in-memory layout."""
    rng = np.random.default_rng(11 + mask)
    N, r = 48, 17.3
    imgs = _images(rng, 3, N)
    for img in imgs:
        y, st = PP.normalise(img, r)
        y = PP.soft_mask(y, r) if mask else y
        out = np.zeros(N * N)
        sref = np.zeros(3)
        R.ref_prep_image(np.ascontiguousarray(io.centred(img)).ravel(), N, r, mask, out, sref)
        np.testing.assert_allclose(io.centred(y).ravel(), out, rtol=0, atol=1e-12)
        np.testing.assert_allclose(st, sref, rtol=1e-13)


@needs_ref
@pytest.mark.parametrize("mask", [0, 1])
def test_preprocessing_chain_matches_reference(mask):
    """The oracle's whole preprocessing of an image -- normalisation, zero
    soft mask, the transform of the image held with its centre at index 0 and
    the pixel gather -- against the reference's own chain: bgMeanStddev /
    softMask (ref_prep_image), then FFT::fw through the vendored FFTW
    (ref_fw_image), gathered at (iCol, iRow mod N)."""
    rng = np.random.default_rng(21 + mask)
    N, r = 48, 17.3
    img = _images(rng, 1, N)
    iCol = rng.integers(0, N // 2 + 1, 300)
    iRow = rng.integers(-N // 2, N // 2, 300)
    dat, _, _ = PP.preprocess(img, r, iCol, iRow, mask=bool(mask), std_n=1.0)
    out = np.zeros(N * N)
    R.ref_prep_image(np.ascontiguousarray(io.centred(img[0])).ravel(), N, r, mask, out, np.zeros(3))
    F = O.ref_fw_image(out.reshape(N, N))
    ref = F[iRow % N, iCol]
    assert np.abs(dat[0] - ref).max() < 1e-12 * np.abs(ref).max()


@needs_ref
def test_remask_matches_reference():
    """oracle/preprocess.py remask against Optimiser::reMaskImg compiled
    (FFT::bw, the softMask mask image, MUL_RL, FFT::fw on the vendored FFTW)."""
    rng = np.random.default_rng(31)
    for N, r in ((32, 9.5), (64, 21.0)):
        F = np.fft.rfft2(rng.standard_normal((N, N)))
        ref = O.ref_remask(F, r)
        got = PP.remask(F[None], r)[0]
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()


def test_preprocessed_pixels_are_the_image_transform():
    """The oracle's pixel data is the transform of the centred image: a unit
    point one pixel right of the centre (inside the mask radius, so the
    background statistics do not change) adds exp(-2 pi i iCol / N) / s."""
    rng = np.random.default_rng(9)
    N, r = 32, 10.0
    iCol, iRow = np.array([0, 3, 5, 1]), np.array([0, -2, 4, -7])
    img0 = rng.standard_normal((1, N, N))
    img1 = img0.copy()
    img1[0, N // 2, N // 2 + 1] += 1.0
    d0, st0, _ = PP.preprocess(img0, r, iCol, iRow, mask=False, std_n=1.0)
    d1, st1, _ = PP.preprocess(img1, r, iCol, iRow, mask=False, std_n=1.0)
    np.testing.assert_array_equal(st0, st1)
    np.testing.assert_allclose((d1 - d0)[0] * st0[0, 1], np.exp(-2j * np.pi * iCol / N),
                               atol=1e-12)


def _thu_line(v, path, mic):
    """One line as Optimiser::saveDatabase prints it (src/Optimiser.cpp:8221)."""
    return ("%18.9lf %18.9lf %18.9lf %18.9lf %18.9lf %18.9lf %18.9lf "
            "                 %s %s %18.9lf %18.9lf "
            "                 %6d %6lu "
            "                 %18.9lf %18.9lf %18.9lf %18.9lf "
            "                 %18.9lf %18.9lf %18.9lf "
            "                 %18.9lf %18.9lf %18.9lf %18.9lf "
            "                 %18.9lf %18.9lf "
            "                 %18.9lf\n").replace("lf", "f").replace("lu", "d") % (
        *v[:7], path, mic, v[9], v[10], int(v[11]), int(v[12]), *v[13:27])


def _thu_rows(rng, n):
    v = rng.uniform(-5, 5, (n, io.THU_COLUMNS))
    v[:, 0] = 300.0
    v[:, io.THU_PATH] = np.nan
    v[:, io.THU_MICROGRAPH] = np.nan
    v[:, io.THU_GROUP] = rng.integers(1, 9, n)
    v[:, io.THU_CLASS] = rng.integers(0, 4, n)
    return np.round(v, 9)


def test_thu_reads_saved_database_lines(tmp_path):
    rng = np.random.default_rng(5)
    v = _thu_rows(rng, 7)
    paths = ["%06d@Particles/stack_%02d.mrcs" % (i + 1, i % 3) for i in range(7)]
    mics = ["Micrographs/mic_%03d.mrc" % i for i in range(7)]
    p = tmp_path / "Meta_Round_001.thu"
    p.write_text("".join(_thu_line(v[i], paths[i], mics[i]) for i in range(7)) + "\n")
    cols, pp, mm = io.read_thu(p)
    np.testing.assert_allclose(cols, v, rtol=0, atol=5e-10, equal_nan=True)
    assert pp == paths and mm == mics
    # ids and the CTF attribute block as the reference reads them (atof / atoi)
    assert cols[:, io.THU_GROUP].astype(int).tolist() == v[:, io.THU_GROUP].astype(int).tolist()


def test_thu_round_trip_and_errors(tmp_path):
    rng = np.random.default_rng(6)
    v = _thu_rows(rng, 5)
    paths = ["%d@a.mrcs" % (i + 1) for i in range(5)]
    mics = ["m.mrc"] * 5
    p = tmp_path / "o.thu"
    io.write_thu(p, v, paths, mics)
    cols, pp, mm = io.read_thu(p)
    np.testing.assert_allclose(cols, v, rtol=0, atol=5e-10, equal_nan=True)
    assert pp == paths and mm == mics
    bad = tmp_path / "bad.thu"
    bad.write_text("300.0 1 2\n")
    with pytest.raises(tg3.TG3Error):
        io.read_thu(bad)
    with pytest.raises(tg3.TG3Error):
        io.write_thu(tmp_path / "x.thu", v, ["has space"] * 5, mics)


@needs_ref
def test_power_spectrum_matches_reference():
    """Shell means of the oracle against the compiled reference's
    powerSpectrum (rint shells, i^2 + j^2 < r^2, the x = 0 column counted on
    both sides)."""
    rng = np.random.default_rng(21)
    N, r = 32, 15
    F = rng.standard_normal((N, N // 2 + 1)) + 1j * rng.standard_normal((N, N // 2 + 1))
    ref = np.zeros(r)
    R.ref_power_spectrum(np.ascontiguousarray(F), N, r, ref)
    np.testing.assert_allclose(PP.power_spectrum(F, r), ref, rtol=1e-13)


def test_spectrum_pixels_are_the_power_spectrum_support():
    rng = np.random.default_rng(22)
    N, r = 32, 15
    F = rng.standard_normal((N, N // 2 + 1)) + 1j * rng.standard_normal((N, N // 2 + 1))
    iCol, iRow = io.spectrum_pixels(N, r)
    u = np.rint(np.sqrt(iCol.astype(float) ** 2 + iRow ** 2)).astype(int)
    assert u.max() == r - 1 and np.all(np.bincount(u) > 0)
    v = np.abs(F[iRow % N, iCol]) ** 2
    np.testing.assert_allclose(np.bincount(u, weights=v) / np.bincount(u),
                               PP.power_spectrum(F, r), rtol=1e-13)


@needs_ref
def test_mkb_real_space_form_is_the_transform_of_the_reference_window():
    """The oracle's MKB_RL (closed form) against the 3-D Fourier transform
    of the reference's own Fourier-space window MKB_FT (compiled, sampled as
    its TabFunction), integrated radially: 4 pi int_0^a MKB_FT(k) sinc(2 k r)
    k^2 dk, compared as ratios to r = 0."""
    from scipy import integrate
    from oracle import reconstruct as RC
    a, alpha, n = 1.9, 15.0, 200000
    tab = np.zeros(n + 1)
    R.ref_mkb_table(a, alpha, a * a, n, tab)       # MKB_FT as a function of k^2
    ft = lambda k: np.interp(k * k, np.linspace(0, a * a, n + 1), tab)

    def rl(r):
        f = lambda k: ft(k) * np.sinc(2 * k * r) * k * k
        return 4 * np.pi * integrate.quad(f, 0, a, limit=400, epsabs=1e-13)[0]

    rs = np.array([0.0, 0.02, 0.05, 0.1, 0.2, 0.3])
    num = np.array([rl(r) for r in rs])
    np.testing.assert_allclose(RC.mkb_rl(rs, a, alpha) / RC.mkb_rl(0.0, a, alpha), num / num[0],
                               rtol=2e-4, atol=1e-7)
