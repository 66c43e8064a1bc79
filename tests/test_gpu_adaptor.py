"""The drop-in adaptor run, not only compiled: interface/Interface.cpp is built
with a C++ driver (tests/adaptor/driver.cpp) against libtg3.so and called
through the reference's own call sequences -- the local expectation
(ExpectPreidx, ExpectLocalIn, ExpectLocalV3D, then per image ExpectLocalP,
ExpectLocalHostA, ExpectLocalRTD, ExpectLocalPreI3D, ExpectLocalM,
ExpectLocalHostF; ExpectLocalFin, ExpectFreeIdx), the same in 2-D mode
(ExpectLocalV2D, ExpectLocalPreI2D) and both InsertFT forms
(single class; multi-class with per-image draw counts nC).  What the caller
receives is compared with the oracle:
- the marginal weights wR, wT as distributions within 2e-3 and the same best
  rotation and translation (the FP32 bar of the other parity tests);
- F, T within 2e-4 of their peaks (trilinear kernel, the reference's GPU
  insertion), O3D to 1e-9 and the counter exactly, the multi-class form
  inserting only draws m < nC[l];
- with a hemisphere of two ranks holding the same data, F and T are summed
  over it (twice the one-rank volumes) and O3D and the counter are not.
Where the reference tree is absent (the GPU machine) the adaptor compiles
against tests/adaptor/Interface.h, a stand-in of the reference's types."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "thunder-refactor-expectation_gb300"


def f32(x):
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.astype(np.complex64).astype(np.complex128)
    return x.astype(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def run(tmp_path_factory):
    d = tmp_path_factory.mktemp("adaptor")
    exe = d / "driver"
    tg3.lib()                       # libtg3.so exists (built by build())
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + str(ROOT / "tests" / "adaptor"),
                        "-I" + str(ROOT / "include"),
                        str(PKG / "interface" / "Interface.cpp"),
                        str(ROOT / "tests" / "adaptor" / "driver.cpp"),
                        "-L" + str(PKG), "-ltg3", "-Wl,-rpath," + str(PKG), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    rng = np.random.default_rng(57)
    box, pf, px, rU = 32, 2, 1.5, 10
    nP, nR, nT, mReco = 6, 60, 9, 3
    rL = synth.config_rL(box, px)
    bm = synth.blob_map(rng, 20, (2.0, 4.0), px, 9.0)
    vol = synth.padded_volume(bm, box, pf).numpy().astype(np.complex64)
    st = synth.make_stack(58, [bm], box, px, pf, rU, rL, nP, 2.0, 0.5)
    qs, ts = synth.local_hypotheses(rng, st.quat_true, st.trans_true, nR, nT, 200.0, 1.0)
    c = dict(box=box, pf=pf, nP=nP, nR=nR, nT=nT, mReco=mReco, vol=vol, st=st,
             dat=st.dat.astype(np.complex64), ctf=st.ctf.astype(np.float32),
             sig=st.sigRcp.astype(np.float32), rot=qs, trans=ts,
             oldR=rng.random((nP, nR)) + 0.5, oldT=rng.random((nP, nT)) + 0.5,
             ins_rot=synth.haar_quaternions(rng, nP * mReco).reshape(nP, mReco, 4),
             ins_trans=rng.uniform(-2, 2, (nP, mReco, 2)), offs=rng.uniform(-0.5, 0.5, (nP, 2)),
             w=(rng.random(nP) + 0.5).astype(np.float32),
             nc=np.array([3, 0, 1, 2, 3, 1], np.int32),
             img2d=synth.class_images_2d([bm], box, pf)[0].cpu().numpy().astype(np.complex64))
    ang = rng.uniform(0, 2 * np.pi, (nP, nR))
    c["rot2d"] = np.stack([np.cos(ang), np.sin(ang)], -1)
    (d / "meta.txt").write_text(f"{box} {pf} {st.K} {nP} {nR} {nT} {mReco}\n")
    for name, a, dt in (("vol", vol, np.complex64), ("icol", st.iCol, np.int32),
                        ("irow", st.iRow, np.int32), ("dat", c["dat"], np.complex64),
                        ("ctf", c["ctf"], np.float32), ("sig", c["sig"], np.float32),
                        ("rot", qs, np.float64), ("trans", ts, np.float64),
                        ("oldR", c["oldR"], np.float64), ("oldT", c["oldT"], np.float64),
                        ("ins_rot", c["ins_rot"], np.float64),
                        ("ins_trans", c["ins_trans"], np.float64),
                        ("offs", c["offs"], np.float64), ("w", c["w"], np.float32),
                        ("nc", c["nc"], np.int32), ("vol2d", c["img2d"], np.complex64),
                        ("rot2d", c["rot2d"], np.float64)):
        np.ascontiguousarray(a, dt).tofile(d / f"{name}.bin")
    outs = {}
    for ranks in (1, 2):
        r = subprocess.run([str(exe), str(d), str(ranks)], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        vd = box * pf
        shape = (vd, vd, vd // 2 + 1)
        o = {k: np.fromfile(d / f"out_{k}.bin", np.float32) for k in ("wC", "wR", "wT")}
        o.update({"2" + k: np.fromfile(d / f"out2_{k}.bin", np.float32)
                  for k in ("wC", "wR", "wT")})
        for form in (1, 2):
            o[f"F{form}"] = np.fromfile(d / f"out_F{form}.bin", np.complex64).reshape(shape)
            o[f"T{form}"] = np.fromfile(d / f"out_T{form}.bin", np.float32).reshape(shape)
            o[f"O{form}"] = np.fromfile(d / f"out_O{form}.bin", np.float64)
            o[f"c{form}"] = int(np.fromfile(d / f"out_c{form}.bin", np.int32)[0])
            o[f"red{form}"] = int(np.fromfile(d / f"out_red{form}.bin", np.int64)[0])
        outs[ranks] = o
    return c, outs


def test_local_sequence_matches_the_oracle(run):
    c, outs = run
    o, st = outs[1], c["st"]
    wR = o["wR"].reshape(c["nP"], c["nR"]).astype(np.float64)
    wT = o["wT"].reshape(c["nP"], c["nT"]).astype(np.float64)
    vol = f32(c["vol"])
    for l in range(c["nP"]):
        ref = O.score_local(vol, c["pf"], st.iCol, st.iRow, c["box"], f32(c["dat"][l]),
                            f32(c["ctf"][l]), f32(c["sig"][l]), f32(c["rot"][l]),
                            f32(c["trans"][l]), c["oldR"][l], c["oldT"][l], 1.0)
        assert np.abs(wR[l] / wR[l].sum() - ref["wR"] / ref["wR"].sum()).max() < 2e-3
        assert np.abs(wT[l] / wT[l].sum() - ref["wT"] / ref["wT"].sum()).max() < 2e-3
        assert np.argmax(wR[l]) == np.argmax(ref["wR"])
        assert np.argmax(wT[l]) == np.argmax(ref["wT"])


def test_local_sequence_2d_matches_the_oracle(run):
    """The 2-D local sequence (ExpectLocalV2D, ExpectLocalPreI2D, in-plane
    rotations) against the oracle's bilinear projection and likelihood."""
    c, outs = run
    o, st = outs[1], c["st"]
    nP, nR, nT = c["nP"], c["nR"], c["nT"]
    wR = o["2wR"].reshape(nP, nR).astype(np.float64)
    wT = o["2wT"].reshape(nP, nT).astype(np.float64)
    img = f32(c["img2d"])
    for l in range(nP):
        P = O.project2d(img, c["rot2d"][l], st.iCol, st.iRow, c["pf"])
        S = O.translate(f32(c["trans"][l]), c["box"], st.iCol, st.iRow)
        X, cc, ss = f32(c["dat"][l]), f32(c["ctf"][l]), f32(c["sig"][l])
        L = np.array([[O.logdvp(X, S[t] * P[r], cc, ss) for t in range(nT)] for r in range(nR)])
        e = np.exp(L - L.max())
        # the marginals of updateSP (or_score_local): wR[r] sums over t with
        # the translation priors, wT[t] over r with the rotation priors
        rR = (e * c["oldT"][l][None, :]).sum(1)
        rT = (e * c["oldR"][l][:, None]).sum(0)
        assert np.abs(wR[l] / wR[l].sum() - rR / rR.sum()).max() < 2e-3
        assert np.abs(wT[l] / wT[l].sum() - rT / rT.sum()).max() < 2e-3
        assert np.argmax(wR[l]) == np.argmax(rR)
        assert np.argmax(wT[l]) == np.argmax(rT)


def _oracle_insert(c, counts):
    st, pf, box = c["st"], c["pf"], c["box"]
    vd = pf * box
    F = np.zeros((vd, vd, vd // 2 + 1), np.complex128)
    T = np.zeros(F.shape)
    O3 = np.zeros(3)
    n = 0
    tab = O.mkb_table(1.9, 15.0, (pf * 1.9) ** 2, 100000)
    for l in range(c["nP"]):
        mats = O.rotmat(c["ins_rot"][l])
        for m in range(counts[l]):
            tt = f32(c["ins_trans"][l, m]) - f32(c["offs"][l])
            img = O.translate_image(f32(c["dat"][l]), -tt[0], -tt[1], box, st.iCol, st.iRow)
            O.insert(F, T, img, f32(c["ctf"][l]), mats[m], float(c["w"][l]), st.iCol * pf,
                     st.iRow * pf, 0, pf * 1.9, tab, (pf * 1.9) ** 2)
            # O3D from the translations as passed (doubles), as the library sums it
            O3 -= mats[m].reshape(3, 3)[:, :2] @ (c["ins_trans"][l, m] - c["offs"][l])
            n += 1
    return F, T, O3, n


@pytest.mark.parametrize("form", [1, 2])
def test_insertft_forms_match_the_oracle(run, form):
    c, outs = run
    o = outs[1]
    counts = [c["mReco"]] * c["nP"] if form == 1 else list(c["nc"])
    F, T, O3, n = _oracle_insert(c, counts)
    assert np.abs(o[f"F{form}"] - F).max() < 2e-4 * np.abs(F).max()
    assert np.abs(o[f"T{form}"] - T).max() < 2e-4 * np.abs(T).max()
    np.testing.assert_allclose(o[f"O{form}"], O3, rtol=0, atol=1e-9)
    assert o[f"c{form}"] == n


@pytest.mark.parametrize("form", [1, 2])
def test_insertft_sums_over_the_hemisphere(run, form):
    c, outs = run
    one, two = outs[1], outs[2]
    vd = c["pf"] * c["box"]
    nvox = vd * vd * (vd // 2 + 1)
    # F (2 floats per voxel) and T summed over the ranks; nothing else
    assert two[f"red{form}"] == 3 * nvox
    # separate runs: the insertion's float atomics may add in another order
    for k in ("F", "T"):
        a, b = two[f"{k}{form}"], 2 * one[f"{k}{form}"]
        assert np.abs(a - b).max() < 1e-6 * np.abs(b).max()
    np.testing.assert_allclose(two[f"O{form}"], one[f"O{form}"], rtol=0, atol=1e-12)
    assert two[f"c{form}"] == one[f"c{form}"]
