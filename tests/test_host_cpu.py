"""CPU-only checks: the C-ABI library loads and exports every declared entry
point, and the host-side input generation follows the reference's rules."""
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from tg3 import synth

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(tg3_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_lists_entry_points():
    names = declared_symbols()
    assert {"tg3_ExpectRotran", "tg3_ExpectProject", "tg3_ExpectGlobal3D", "tg3_InsertFT",
            "tg3_local_phase_d", "tg3_resample"} <= names


def test_library_exports_every_declared_symbol():
    import ctypes
    import tg3
    if not tg3.LIB_PATH.exists():
        from tg3 import build
        build.build()
    lib = ctypes.CDLL(str(tg3.LIB_PATH))
    names = declared_symbols()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(tg3.EXPORTS) == names
    # calls that need no GPU
    tg3.lib()
    assert tg3.version().startswith("tg3")
    assert tg3.lib().tg3_status_string(tg3.ERR_ARG) == b"invalid argument"


def test_pixel_index_matches_oracle():
    for box, px, rU in [(64, 1.5, 16), (256, 1.1, 80), (192, 1.3, 40), (24, 1.0, 7.5)]:
        rL = synth.config_rL(box, px)
        a = synth.pixel_index(box, rU, rL)
        b = O.pixel_index(box, rU, rL)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


def test_pixel_counts_of_the_configurations():
    # K of each benchmark configuration under the reference's selection rule
    for box, px, rU, K in [(64, 1.5, 16, 375), (256, 1.1, 80, 9930), (256, 1.1, 120, 22422),
                           (192, 1.3, 40, 2452), (192, 1.3, 56, 4844), (192, 1.3, 72, 8026),
                           (192, 1.3, 96, 14324)]:
        assert len(synth.pixel_index(box, rU, synth.config_rL(box, px))[0]) == K


def test_quaternion_matrices_match_oracle():
    q = synth.haar_quaternions(np.random.default_rng(0), 50)
    np.testing.assert_allclose(synth.quat_to_mat(q), O.rotmat(q), atol=1e-15)
    R = synth.quat_to_mat(q)
    np.testing.assert_allclose(R @ R.transpose(0, 2, 1), np.broadcast_to(np.eye(3), R.shape),
                               atol=1e-12)


def test_global_rotation_grid():
    hp = synth.healpix_ring_centres(4)
    assert hp.shape == (192, 2)
    z = np.cos(hp[:, 0])
    # equal-area pixels: the z histogram of centres is symmetric
    np.testing.assert_allclose(np.sort(z), -np.sort(z)[::-1], atol=1e-12)
    q = synth.global_rotations(4, 36)
    assert q.shape == (6912, 4)
    np.testing.assert_allclose(np.linalg.norm(q, axis=1), 1, atol=1e-12)
    assert len(synth.global_translations(3, 1.0)) == 49


def test_vmf_concentration():
    rng = np.random.default_rng(1)
    mean = synth.haar_quaternions(rng, 1)[0]
    s = synth.vmf_quaternions(rng, mean, 200.0, 4000)
    c = np.abs(s @ mean)
    # E[1 - mu.x] ~ (p - 1) / (2 kappa) for large kappa on S^3
    assert abs(np.mean(1 - c) - 3 / 400) < 1e-3


def test_ctf_vectorised_matches_oracle():
    rng = np.random.default_rng(2)
    iCol, iRow, _, _ = synth.pixel_index(64, 16, 0)
    attr = synth.ctf_attrs(rng, 5)
    np.testing.assert_allclose(synth.ctf_values(attr, 1.5, 64, iCol, iRow),
                               O.ctf(attr, 1.5, 64, iCol, iRow), atol=1e-12)


def test_2d_particle_generator_matches_oracle_projection():
    """The benchmark's torch generator of 2-D particles samples the class
    images as the oracle's 2-D projection does (bilinear, Friedel mirror,
    wrapped rows)."""
    import torch
    rng = np.random.default_rng(5)
    box, pf, px = 24, 2, 1.5
    maps = [synth.blob_map(rng, 12, (1.5, 3.0), px, 8.0) for _ in range(2)]
    imgs = synth.class_images_2d(maps, box, pf)
    iCol, iRow = synth.pixel_index(box, 10, synth.config_rL(box, px))[:2]
    ang = rng.uniform(0, 2 * np.pi, 5)
    rot = np.stack([np.cos(ang), np.sin(ang)], 1)
    k = np.array([0, 1, 1, 0, 1])
    got = synth.sample_2d(imgs, torch.as_tensor(k), torch.as_tensor(rot), iCol, iRow, pf).numpy()
    for r in range(5):
        ref = O.project2d(imgs[k[r]].numpy().astype(np.complex128), rot[r:r + 1], iCol, iRow, pf)[0]
        np.testing.assert_allclose(got[r], ref, rtol=0, atol=2e-5 * np.abs(ref).max())


def test_blob_volume_is_hermitian_on_x0_plane():
    rng = np.random.default_rng(3)
    bm = synth.blob_map(rng, 5, (2.0, 4.0), 1.5, 5.0)
    v = synth.padded_volume(bm, 16, 2).numpy()
    n = v.shape[0]
    for y in range(1, n // 2):
        for z in range(1, n // 2):
            assert np.isclose(v[z, y, 0], np.conj(v[n - z, n - y, 0]), atol=1e-10)


REF = O.REF_TREE


@pytest.mark.skipif(not (REF / "gpu" / "interface" / "Interface.h").exists(),
                    reason="reference sources unavailable")
def test_dropin_adaptor_compiles_against_reference_interface(tmp_path):
    """interface/Interface.cpp defines the E-step and insertion entry points
    with the exact signatures of the reference's gpu/interface/Interface.h."""
    import subprocess
    from oracle import oracle as Oo
    Oo.build_ref()   # provides the GSL/FFTW header links and the MPI stand-in
    incs = ["-I" + str(ROOT / "oracle" / "_ref" / "inc"), "-I" + str(ROOT / "oracle" / "ref")]
    incs += ["-I" + str(p) for p in (REF / "include").rglob("*") if p.is_dir()]
    incs += ["-I" + str(REF / "include"), "-I" + str(REF / "gpu" / "interface"),
             "-I" + str(REF / "gpu" / "include"), "-I" + str(REF / "external" / "Eigen3"),
             "-I" + str(REF / "external" / "boost"), "-I" + str(REF / "external" / "easylogging"),
             "-I" + str(ROOT / "include"), "-I/usr/local/cuda/include"]
    obj = tmp_path / "iface.o"
    r = subprocess.run(["g++", "-std=c++11", "-c", "-w", "-DSINGLE_PRECISION", "-DGPU_VERSION",
                        *incs, str(ROOT / "thunder-refactor-expectation_gb300" / "interface" /
                                   "Interface.cpp"), "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    syms = subprocess.run(["nm", "-C", str(obj)], capture_output=True, text=True).stdout
    for name in ("ExpectRotran(", "ExpectProject(", "ExpectGlobal3D(", "ExpectLocalM(",
                 "ExpectLocalPreI3D(", "InsertFT(Volume&", "getAviDevice("):
        assert any(" T " in ln and name in ln for ln in syms.splitlines()), name


def test_binding_signatures_match_header():
    """The ctypes argument lists agree with the header's parameter counts."""
    import tg3
    if not tg3.LIB_PATH.exists():
        from tg3 import build
        build.build()
    L = tg3.lib()
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "thunder_gb300.h").read_text(), flags=re.S)
    for m in re.finditer(r"\b(tg3_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        name, params = m.group(1), m.group(2).strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(getattr(L, name).argtypes) == n, (name, n, len(getattr(L, name).argtypes))


def test_symmetrize_offsets_is_host_arithmetic():
    """tg3_SymmetrizeO (Reconstructor::symmetrizeO): O + sum_s R_s O over the
    elements besides the identity, counter times 1 + nSym -- host arithmetic,
    so it runs without a device; against numpy for C4 about z."""
    import ctypes
    import tg3
    sys_path = Path(__file__).resolve().parent / "golden"
    import sys
    sys.path.insert(0, str(sys_path))
    from make_golden import symmetry_elements
    c4, _ = symmetry_elements()
    o = np.array([1.5, -0.25, 2.0])
    got = o.copy()
    cnt = np.array([7], np.int32)
    tg3.check(tg3.lib().tg3_SymmetrizeO(tg3.ptr(got), tg3.ptr(cnt),
                                        tg3.ptr(np.ascontiguousarray(c4.reshape(-1, 9))), len(c4)))
    want = o + sum(m @ o for m in c4)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-12)
    assert cnt[0] == 7 * 4
    # C4 about z: the x, y parts cancel, z adds up four times
    np.testing.assert_allclose(got, [0.0, 0.0, 8.0], atol=1e-12)
