"""GPU parity: every CUDA stage of the E-step and the insertion, called
through the C ABI (libtg3.so), against the double-precision oracle on the
same seeded inputs.  The oracle receives the float32-rounded inputs the GPU
sees, so the differences measured are the GPU's arithmetic only.

Tolerances (FP32 plain path, from the acceptance bars): log-likelihoods
within 1e-4 relative; marginal weights compared after normalisation within
2e-3 absolute on the distribution; projections within 1e-5 of the slice's
peak magnitude; resampling bit-exact; insertion FSC >= 0.999."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def f32(x):
    """float32-rounded copy in float64 (complex128 for complex)."""
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.astype(np.complex64).astype(np.complex128)
    return x.astype(np.float32).astype(np.float64)


def dev(x, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(x))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(DEV).contiguous()


@pytest.fixture(scope="module")
def small():
    rng = np.random.default_rng(11)
    box, pf, px = 32, 2, 1.5
    rU = 12
    iCol, iRow, iSig, _ = synth.pixel_index(box, rU, synth.config_rL(box, px))
    bm = synth.blob_map(rng, 20, (2.0, 4.0), px, 9.0)
    vol = synth.padded_volume(bm, box, pf).numpy()
    vol32 = vol.astype(np.complex64)
    st = synth.make_stack(5, [bm], box, px, pf, rU, synth.config_rL(box, px), 48, 2.0, 0.5)
    return dict(rng=rng, box=box, pf=pf, px=px, iCol=iCol, iRow=iRow, vol=f32(vol32),
                vol32=vol32, st=st)


@pytest.fixture(scope="module")
def ctx(small):
    c = tg3.Context(0)
    c.set_volume(0, torch.as_tensor(small["vol32"]).to(DEV), small["pf"])
    c.set_pixels(small["iCol"], small["iRow"], small["box"])
    yield c
    c.close()


def test_rotmat_translate_ctf(small):
    rng = small["rng"]
    q = synth.haar_quaternions(rng, 33)
    mat = torch.empty((33, 9), dtype=torch.float64, device=DEV)
    dq = dev(q)
    tg3.check(tg3.lib().tg3_rotmat_d(tg3.ptr(dq), 33, tg3.ptr(mat), None))
    torch.cuda.synchronize()
    np.testing.assert_allclose(mat.cpu().numpy(), O.rotmat(q).reshape(-1, 9), rtol=0, atol=1e-15)

    iCol, iRow, K = small["iCol"], small["iRow"], len(small["iCol"])
    t = rng.uniform(-8, 8, (7, 2))
    out = torch.empty((7, K, 2), dtype=torch.float32, device=DEV)
    dt, dc, dr = dev(t), dev(iCol), dev(iRow)
    tg3.check(tg3.lib().tg3_translate_d(tg3.ptr(dt), 7, small["box"], tg3.ptr(dc),
                                        tg3.ptr(dr), K, tg3.ptr(out), None))
    torch.cuda.synchronize()
    S = out.cpu().numpy().astype(np.float64)
    S = S[..., 0] + 1j * S[..., 1]
    np.testing.assert_allclose(S, O.translate(f32(t), small["box"], iCol, iRow), atol=2e-6)

    attr = synth.ctf_attrs(rng, 4)
    cout = torch.empty((4, K), dtype=torch.float32, device=DEV)
    da = dev(attr, torch.float32)
    tg3.check(tg3.lib().tg3_ctf_d(tg3.ptr(da), 4, small["px"], small["box"],
                                  tg3.ptr(dc), tg3.ptr(dr), K, tg3.ptr(cout), None))
    torch.cuda.synchronize()
    ref = O.ctf(f32(attr), small["px"], small["box"], iCol, iRow)
    np.testing.assert_allclose(cout.cpu().numpy(), ref, atol=5e-4)


def test_project(small, ctx):
    rng = small["rng"]
    q = synth.haar_quaternions(rng, 64)
    mat = O.rotmat(q).reshape(-1, 9)
    K = len(small["iCol"])
    out = torch.empty((64, K, 2), dtype=torch.float32, device=DEV)
    ctx.project(0, dev(mat), 64, out)
    ctx.sync()
    P = out.cpu().numpy().astype(np.float64)
    P = P[..., 0] + 1j * P[..., 1]
    ref = O.project(small["vol"], mat, small["iCol"], small["iRow"], small["pf"])
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert np.max(np.abs(P - ref) / scale) < 1e-5


def test_project_forms(small, ctx):
    """The projection forms (TG3_OPT_PROJECT_FORM: 0 lane pair, 1 one lane per
    pixel, 2 the same with a computed block index, 3 / 4 lane pairs sharing
    whole-block loads) against the oracle, and against each other: the same
    corner sums in the same order, so the samples agree to within one
    rounding of a sum's contraction, and forms differing only in how the
    block index is found (1 and 2, 3 and 4) exactly."""
    rng = small["rng"]
    q = synth.haar_quaternions(rng, 40)
    mat = O.rotmat(q).reshape(-1, 9)
    K = len(small["iCol"])
    res = {}
    try:
        for form in (0, 1, 2, 3, 4):
            ctx.set_option(tg3.OPT_PROJECT_FORM, form)
            out = torch.empty((40, K, 2), dtype=torch.float32, device=DEV)
            ctx.project(0, dev(mat), 40, out)
            ctx.sync()
            P = out.cpu().numpy().astype(np.float64)
            res[form] = P[..., 0] + 1j * P[..., 1]
    finally:
        ctx.set_option(tg3.OPT_PROJECT_FORM, 4)
    ref = O.project(small["vol"], mat, small["iCol"], small["iRow"], small["pf"])
    scale = np.abs(ref).max(axis=1, keepdims=True)
    for form in (0, 1, 2, 3, 4):
        assert np.max(np.abs(res[form] - ref) / scale) < 1e-5
    assert np.max(np.abs(res[0] - res[1]) / scale) < 1e-6
    assert np.max(np.abs(res[0] - res[3]) / scale) < 1e-6
    np.testing.assert_array_equal(res[1], res[2])
    np.testing.assert_array_equal(res[3], res[4])


@pytest.mark.parametrize("group", [4, 16])
def test_project_groups(small, ctx, group):
    """Projection form 4 with 4 or 16 rotations a CTA (TG3_OPT_PROJECT_GROUP)
    against the default 8: the same samples, bit for bit, 37 rotations
    leaving partial groups."""
    rng = small["rng"]
    q = synth.haar_quaternions(rng, 37)
    mat = O.rotmat(q).reshape(-1, 9)
    K = len(small["iCol"])
    res = {}
    try:
        for gr in (8, group):
            ctx.set_option(tg3.OPT_PROJECT_GROUP, gr)
            out = torch.empty((37, K, 2), dtype=torch.float32, device=DEV)
            ctx.project(0, dev(mat), 37, out)
            ctx.sync()
            res[gr] = out.cpu().numpy()
    finally:
        ctx.set_option(tg3.OPT_PROJECT_GROUP, 8)
    np.testing.assert_array_equal(res[8], res[group])


def test_local_phase_project_forms(small, ctx):
    """The split-bf16 local phase with either projection form: likelihoods
    within 1e-6 relative of each other (the bf16 split of equal samples is
    equal; the norms' pixel sums run in another order)."""
    nP, nR, nT = 3, 200, 30
    d = _local_inputs(small, nP, nR, nT, 13)
    res = {}
    try:
        for form in (0, 2, 4):
            ctx.set_option(tg3.OPT_PROJECT_FORM, form)
            o = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                     wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                     wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                     base=torch.empty(nP, dtype=torch.float64, device=DEV),
                     dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
            ctx.local_phase(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]),
                            dev(d["qs"]), dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]),
                            dev(d["pwC"]), None, o["wC"], o["wR"], o["wT"], o["base"], o["dvp"],
                            tg3.SCORE_BF16X3)
            ctx.sync()
            res[form] = {k: v.cpu().numpy() for k, v in o.items()}
    finally:
        ctx.set_option(tg3.OPT_PROJECT_FORM, 4)
    a = res[0]["dvp"].astype(np.float64)
    for form in (2, 4):
        b = res[form]["dvp"].astype(np.float64)
        assert np.max(np.abs(a - b)) < 1e-6 * np.abs(a).max()


def test_expect_project_host(small):
    rng = small["rng"]
    q = synth.haar_quaternions(rng, 10)
    mat = np.ascontiguousarray(O.rotmat(q).reshape(-1, 9))
    K = len(small["iCol"])
    rotP = np.zeros((10, K), np.complex64)
    vol = np.ascontiguousarray(small["vol32"])
    tg3.check(tg3.lib().tg3_ExpectProject(tg3.ptr(vol), tg3.ptr(rotP), tg3.ptr(mat),
                                          tg3.ptr(np.ascontiguousarray(small["iCol"])),
                                          tg3.ptr(np.ascontiguousarray(small["iRow"])), 10,
                                          small["pf"], 1, vol.shape[0], K))
    ref = O.project(small["vol"], mat, small["iCol"], small["iRow"], small["pf"])
    assert np.max(np.abs(rotP - ref)) < 1e-5 * np.abs(ref).max()


def _local_inputs(small, nP, nR, nT, seed):
    rng = np.random.default_rng(seed)
    st = small["st"]
    K = st.K
    qs, ts = synth.local_hypotheses(rng, st.quat_true[:nP], st.trans_true[:nP], nR, nT, 200.0, 1.0)
    pwR = rng.random((nP, nR)) + 0.5
    pwT = rng.random((nP, nT)) + 0.5
    pwC = np.ones(nP)
    return dict(qs=qs, ts=ts, pwR=pwR, pwT=pwT, pwC=pwC, dat=st.dat[:nP].astype(np.complex64),
                ctf=st.ctf[:nP].astype(np.float32), sig=st.sigRcp[:nP].astype(np.float32), K=K)


@pytest.mark.parametrize("precision,shape", [
    (tg3.SCORE_FP32, (4, 96, 21)), (tg3.SCORE_BF16X3, (4, 96, 21)),
    (tg3.SCORE_FP32, (3, 300, 100)), (tg3.SCORE_BF16X3, (3, 300, 100))])
def test_local_phase(small, ctx, precision, shape):
    nP, nR, nT = shape
    d = _local_inputs(small, nP, nR, nT, 3)
    outs = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                base=torch.empty(nP, dtype=torch.float64, device=DEV),
                dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
    ctx.local_phase(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]), dev(d["qs"]),
                    dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]), dev(d["pwC"]), None,
                    outs["wC"], outs["wR"], outs["wT"], outs["base"], outs["dvp"], precision)
    ctx.sync()
    g = {k: v.cpu().numpy() for k, v in outs.items()}
    for l in range(nP):
        r = O.score_local(small["vol"], small["pf"], small["iCol"], small["iRow"], small["box"],
                          f32(d["dat"][l]), f32(d["ctf"][l]), f32(d["sig"][l]), f32(d["qs"][l]),
                          f32(d["ts"][l]), d["pwR"][l], d["pwT"][l], 1.0)
        rel = np.abs(g["dvp"][l] - r["dvp"]) / np.abs(r["dvp"])
        assert rel.max() < 1e-4, rel.max()
        assert abs(g["base"][l] - r["base"]) / abs(r["base"]) < 1e-4
        assert np.argmax(g["dvp"][l]) == np.argmax(r["dvp"])
        # weights relative to each one's own baseline: compare normalised forms
        gw = g["wR"][l] / g["wR"][l].sum()
        rw = r["wR"] / r["wR"].sum()
        assert np.abs(gw - rw).max() < 2e-3
        gt = g["wT"][l] / g["wT"][l].sum()
        rt = r["wT"] / r["wT"].sum()
        assert np.abs(gt - rt).max() < 2e-3
        # wC against the same baseline shift
        wc_ref = r["wC"] * np.exp(r["base"] - g["base"][l])
        assert abs(g["wC"][l] - wc_ref) / wc_ref < 5e-2


def test_expect_global3d_two_classes(small):
    rng = np.random.default_rng(17)
    st = small["st"]
    K = st.K
    nImg, nR, nT, nK = 9, 40, 9, 2
    q = synth.haar_quaternions(rng, nR)
    mat = O.rotmat(q).reshape(-1, 9)
    vols = [small["vol"], f32(small["vol32"] * np.complex64(0.8))]
    trans = synth.global_translations(1, 1.0)
    traP = O.translate(f32(trans), small["box"], small["iCol"], small["iRow"]).astype(np.complex64)
    pR = rng.random(nR)
    pT = rng.random(nT)
    dat = st.dat[:nImg].astype(np.complex64)
    ctf = st.ctf[:nImg].astype(np.float32)
    sig = st.sigRcp[:nImg].astype(np.float32)
    wC = np.zeros(nImg * nK, np.float32)
    wR = np.zeros(nImg * nK * nR, np.float32)
    wT = np.zeros(nImg * nK * nT, np.float32)
    bL = np.zeros(nImg, np.float32)
    state = None
    for k in range(nK):
        rotP = O.project(vols[k], mat, small["iCol"], small["iRow"], small["pf"]).astype(np.complex64)
        tg3.check(tg3.lib().tg3_ExpectGlobal3D(
            tg3.ptr(rotP), tg3.ptr(traP), tg3.ptr(dat), tg3.ptr(ctf), tg3.ptr(sig), tg3.ptr(wC),
            tg3.ptr(wR), tg3.ptr(wT), tg3.ptr(pR), tg3.ptr(pT), tg3.ptr(bL), k, nK, nR, nT, K,
            nImg))
        state = O.score_global(f32(rotP), f32(traP), f32(dat), f32(ctf), f32(sig), pR, pT, k, nK,
                               state=None if state is None else (state["wC"], state["wR"],
                                                                 state["wT"], state["baseL"]),
                               want_dvp=False)
    assert np.abs(bL - state["baseL"]).max() / np.abs(state["baseL"]).max() < 1e-4
    for l in range(nImg):
        shift = np.exp(state["baseL"][l] - bL[l])
        a = wC[l * nK:(l + 1) * nK]
        b = state["wC"][l * nK:(l + 1) * nK] * shift
        np.testing.assert_allclose(a / a.sum(), b / b.sum(), atol=2e-3)
        a = wR[l * nK * nR:(l + 1) * nK * nR]
        b = state["wR"][l * nK * nR:(l + 1) * nK * nR] * shift
        np.testing.assert_allclose(a / a.sum(), b / b.sum(), atol=2e-3)


@pytest.mark.parametrize("n,n_out,peak", [(1000, 1000, np.nan), (777, 500, 0.05), (50, 80, 0.0)])
def test_resample_bit_exact(n, n_out, peak):
    rng = np.random.default_rng(n)
    nP = 6
    u = np.exp(3 * rng.standard_normal((nP, n)))
    u[:, rng.integers(0, n, 5)] = 0.0
    w = rng.random((nP, n))
    perm = np.stack([rng.permutation(n) for _ in range(nP)]).astype(np.int32)
    u0 = rng.random(nP) / n_out
    peaks = np.full(nP, peak)
    src = np.zeros((nP, n_out), np.int32)
    wout = np.zeros((nP, n_out))
    top = np.zeros(nP, np.int32)
    tg3.check(tg3.lib().tg3_resample(nP, n, tg3.ptr(u), tg3.ptr(w), tg3.ptr(perm), tg3.ptr(u0),
                                     tg3.ptr(peaks), n_out, tg3.ptr(src), tg3.ptr(wout),
                                     tg3.ptr(top)))
    for b in range(nP):
        pf = O.peak_factor_r(u[b]) if np.isnan(peak) else peak
        s_ref, w_ref, top_ref = O.resample(u[b], w[b], perm[b], u0[b], pf, n_out)
        assert np.array_equal(src[b], s_ref)
        assert np.array_equal(wout[b], w_ref)
        assert top[b] == top_ref


def test_resample_rejects_bad_permutation():
    n = 10
    u = np.ones(n)
    w = np.ones(n)
    perm = np.arange(n, dtype=np.int32)
    perm[3] = 99
    u0 = np.array([0.01])
    src = np.zeros(n, np.int32)
    wout = np.zeros(n)
    top = np.zeros(1, np.int32)
    st = tg3.lib().tg3_resample(1, n, tg3.ptr(u), tg3.ptr(w), tg3.ptr(perm), tg3.ptr(u0), None,
                                n, tg3.ptr(src), tg3.ptr(wout), tg3.ptr(top))
    assert st == tg3.ERR_ARG


@pytest.mark.parametrize("kernel,gather", [(tg3.KERNEL_MKB, 0), (tg3.KERNEL_MKB, 1),
                                           (tg3.KERNEL_TRILINEAR, 0)],
                         ids=["mkb-scatter", "mkb-gather", "trilinear"])
def test_insert(small, kernel, gather):
    rng = np.random.default_rng(23)
    st = small["st"]
    K, pf, box = st.K, small["pf"], small["box"]
    vdim = pf * box
    nP = 12
    q = synth.haar_quaternions(rng, nP)
    t = rng.uniform(-2, 2, (nP, 2))
    off = rng.uniform(-0.5, 0.5, (nP, 2))
    w = rng.uniform(0.5, 1.5, nP).astype(np.float32)
    dat = st.dat[:nP].astype(np.complex64)
    ctf = st.ctf[:nP].astype(np.float32)
    c = tg3.Context(0)
    try:
        c.set_pixels(small["iCol"], small["iRow"], box)
        c.set_option(tg3.OPT_INSERT_GATHER, gather)
        c.insert_begin(vdim, pf)
        O3D = torch.zeros(3, dtype=torch.float64, device=DEV)
        cnt = torch.zeros(1, dtype=torch.int32, device=DEV)
        c.insert(nP, dev(dat), dev(ctf), dev(q), dev(t), dev(off), dev(w), kernel, O3D, cnt)
        F = torch.empty((vdim, vdim, vdim // 2 + 1, 2), dtype=torch.float32, device=DEV)
        T = torch.empty((vdim, vdim, vdim // 2 + 1), dtype=torch.float32, device=DEV)
        c.insert_read(F, T)
        c.sync()
        Fg = F.cpu().numpy().astype(np.float64)
        Fg = Fg[..., 0] + 1j * Fg[..., 1]
        Tg = T.cpu().numpy().astype(np.float64)
        assert int(cnt.item()) == nP
    finally:
        c.close()
    Fr = np.zeros((vdim, vdim, vdim // 2 + 1), np.complex128)
    Tr = np.zeros(Fr.shape)
    tab = O.mkb_table(1.9, 15.0, (pf * 1.9) ** 2, 100000)
    mats = O.rotmat(q)
    Or = np.zeros(3)
    for l in range(nP):
        tt = f32(t[l]) - f32(off[l])
        img = O.translate_image(f32(dat[l]), -tt[0], -tt[1], box, small["iCol"], small["iRow"])
        O.insert(Fr, Tr, img, f32(ctf[l]), mats[l], float(w[l]), small["iCol"] * pf,
                 small["iRow"] * pf, kernel, pf * 1.9, tab, (pf * 1.9) ** 2)
        Or -= mats[l] @ np.array([t[l, 0] - off[l, 0], t[l, 1] - off[l, 1], 0.0])
    np.testing.assert_allclose(O3D.cpu().numpy(), Or, rtol=1e-9, atol=1e-9)
    # volume agreement: relative error and FSC over the shells that hold data
    scale = np.abs(Fr).max()
    assert np.abs(Fg - Fr).max() < 2e-4 * scale
    assert np.abs(Tg - Tr).max() < 2e-4 * np.abs(Tr).max()
    rmax = int(12 * pf)
    f = O.fsc(Fg, Fr, rmax)
    assert f[1:].min() >= 0.999, f


def test_insertft_host(small):
    rng = np.random.default_rng(29)
    st = small["st"]
    K, pf, box = st.K, small["pf"], small["box"]
    vdim = pf * box
    nImg, mReco = 5, 3
    quats = synth.haar_quaternions(rng, nImg * mReco)
    trans = rng.uniform(-2, 2, (nImg * mReco, 2))
    offS = rng.uniform(-0.5, 0.5, (nImg, 2))
    w = (np.ones(nImg) / mReco).astype(np.float32)
    F = np.zeros((vdim, vdim, vdim // 2 + 1), np.complex64)
    F[1, 2, 3] = 1 + 2j       # accumulated into, not overwritten
    T = np.zeros((vdim, vdim, vdim // 2 + 1), np.float32)
    O3D = np.zeros(3)
    counter = np.zeros(1, np.int32)
    dat = np.ascontiguousarray(st.dat[:nImg].astype(np.complex64))
    ctf = np.ascontiguousarray(st.ctf[:nImg].astype(np.float32))
    sig = np.ascontiguousarray(st.sigRcp[:nImg].astype(np.float32))
    # the reconstructor's padded pixel indices, as the reference passes them
    iColPad = np.ascontiguousarray(small["iCol"] * pf, np.int32)
    iRowPad = np.ascontiguousarray(small["iRow"] * pf, np.int32)
    tg3.check(tg3.lib().tg3_InsertFT(
        tg3.ptr(F), tg3.ptr(T), tg3.ptr(O3D), tg3.ptr(counter), tg3.ptr(dat), tg3.ptr(ctf),
        tg3.ptr(sig), None, tg3.ptr(offS), tg3.ptr(w), tg3.ptr(quats), tg3.ptr(trans), None,
        tg3.ptr(iColPad), tg3.ptr(iRowPad),
        small["px"], 0, pf, K, mReco, box, vdim, nImg, tg3.KERNEL_TRILINEAR))
    assert counter[0] == nImg * mReco
    Fr = np.zeros(F.shape, np.complex128)
    Fr[1, 2, 3] = 1 + 2j
    Tr = np.zeros(T.shape)
    tab = O.mkb_table(1.9, 15.0, (pf * 1.9) ** 2, 100000)
    mats = O.rotmat(quats)
    for l in range(nImg):
        for m in range(mReco):
            d = l * mReco + m
            tt = f32(trans[d]) - f32(offS[l])
            img = O.translate_image(f32(dat[l]), -tt[0], -tt[1], box, small["iCol"], small["iRow"])
            O.insert(Fr, Tr, img, f32(ctf[l]), mats[d], float(w[l]), small["iCol"] * pf,
                     small["iRow"] * pf, 0, pf * 1.9, tab, (pf * 1.9) ** 2)
    assert np.abs(F - Fr).max() < 2e-4 * np.abs(Fr).max()
    assert np.abs(T - Tr).max() < 2e-4 * np.abs(Tr).max()


def test_expect_local3d_host(small):
    st = small["st"]
    d = _local_inputs(small, 1, 64, 16, 31)
    vol = np.ascontiguousarray(small["vol32"])
    h = tg3.ctypes.c_void_p()
    tg3.check(tg3.lib().tg3_volume_create(tg3.ctypes.byref(h), tg3.ptr(vol), vol.shape[0],
                                          small["pf"]))
    try:
        wC = np.zeros(1, np.float32)
        wR = np.zeros(64, np.float32)
        wT = np.zeros(16, np.float32)
        dvp = np.zeros((64, 16), np.float32)
        bl = np.zeros(1, np.float32)
        q = np.ascontiguousarray(d["qs"][0])
        t = np.ascontiguousarray(d["ts"][0])
        tg3.check(tg3.lib().tg3_ExpectLocal3D(
            h, tg3.ptr(np.ascontiguousarray(d["dat"][0])), tg3.ptr(np.ascontiguousarray(d["ctf"][0])),
            tg3.ptr(np.ascontiguousarray(d["sig"][0])), tg3.ptr(np.ascontiguousarray(small["iCol"])),
            tg3.ptr(np.ascontiguousarray(small["iRow"])), st.K, small["box"], tg3.ptr(q), 64,
            tg3.ptr(t), 16, tg3.ptr(np.ascontiguousarray(d["pwR"][0])),
            tg3.ptr(np.ascontiguousarray(d["pwT"][0])), 1.0, tg3.ptr(wC), tg3.ptr(wR), tg3.ptr(wT),
            tg3.ptr(dvp), tg3.ptr(bl)))
    finally:
        tg3.lib().tg3_volume_destroy(h)
    r = O.score_local(small["vol"], small["pf"], small["iCol"], small["iRow"], small["box"],
                      f32(d["dat"][0]), f32(d["ctf"][0]), f32(d["sig"][0]), f32(q), f32(t),
                      d["pwR"][0], d["pwT"][0], 1.0)
    assert (np.abs(dvp - r["dvp"]) / np.abs(r["dvp"])).max() < 1e-4
    np.testing.assert_allclose(wR / wR.sum(), r["wR"] / r["wR"].sum(), atol=2e-3)


def test_bad_geometry_rejected(small):
    c = tg3.Context(0)
    try:
        c.set_volume(0, torch.as_tensor(small["vol32"]).to(DEV), small["pf"])
        # a pixel at the image edge cannot be sampled from this volume with margin
        big = np.array([0, 16], np.int32)
        c.set_pixels(big, np.array([16, 0], np.int32), small["box"])
        out = torch.empty((1, 2, 2), dtype=torch.float32, device=DEV)
        with pytest.raises(tg3.TG3Error) as e:
            c.project(0, dev(np.eye(3).reshape(1, 9)), 1, out)
        assert e.value.status == tg3.ERR_ARG
    finally:
        c.close()


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3])
@pytest.mark.parametrize("shape", [(40, 70), (5, 1024)])
def test_global_scan(small, ctx, precision, shape):
    """Device global scan (shared rotations x translations for many images)
    against the oracle's doGlobalSearch restatement.  40 images x 70
    rotations: 360 columns, two split-bf16 column tiles; 5 images x 1,024
    rotations: so few images that each image's rotations are weighed by
    several CTAs and folded (k_merge_chunks)."""
    rng = np.random.default_rng(41)
    st = small["st"]
    nImg, nR = shape
    nT = 9
    q = synth.haar_quaternions(rng, nR)
    mat = np.ascontiguousarray(O.rotmat(q).reshape(-1, 9))
    trans = synth.global_translations(1, 1.0)
    pR = rng.random(nR) + 0.5
    pT = rng.random(nT) + 0.5
    dat = st.dat[:nImg].astype(np.complex64)
    ctf = st.ctf[:nImg].astype(np.float32)
    sig = st.sigRcp[:nImg].astype(np.float32)
    o = dict(wC=torch.empty(nImg, dtype=torch.float64, device=DEV),
             wR=torch.empty((nImg, nR), dtype=torch.float64, device=DEV),
             wT=torch.empty((nImg, nT), dtype=torch.float64, device=DEV),
             base=torch.empty(nImg, dtype=torch.float64, device=DEV),
             dvp=torch.empty((nImg, nR, nT), dtype=torch.float32, device=DEV))
    ctx.global_scan(0, nImg, nR, nT, dev(dat), dev(ctf), dev(sig), dev(mat), dev(trans),
                    dev(pR), dev(pT), o["wC"], o["wR"], o["wT"], o["base"], o["dvp"], precision)
    ctx.sync()
    g = {k: v.cpu().numpy() for k, v in o.items()}
    rotP = O.project(small["vol"], mat, small["iCol"], small["iRow"], small["pf"])
    traP = O.translate(f32(trans), small["box"], small["iCol"], small["iRow"])
    r = O.score_global(rotP, traP, f32(dat), f32(ctf), f32(sig), pR, pT)
    rel = np.abs(g["dvp"] - r["dvp"]) / np.abs(r["dvp"])
    assert rel.max() < 1e-4, rel.max()
    for l in range(nImg):
        assert np.argmax(g["dvp"][l]) == np.argmax(r["dvp"][l])
        a = g["wR"][l] / g["wR"][l].sum()
        b = r["wR"][l * nR:(l + 1) * nR]
        np.testing.assert_allclose(a, b / b.sum(), atol=2e-3)
        a = g["wT"][l] / g["wT"][l].sum()
        b = r["wT"][l * nT:(l + 1) * nT]
        np.testing.assert_allclose(a, b / b.sum(), atol=2e-3)


@pytest.mark.parametrize("form", [(0, 1, 64), (128, 0, 64), (128, 1, 64), (64, 1, 64),
                                  (0, 0, 32), (0, 1, 32)])
def test_global_scan_tile_forms(small, ctx, form):
    """The split-bf16 global scan's cross term with a narrower column tile
    (TG3_OPT_SCAN_TILE_N), on CTA pairs that share each column tile by TMA
    multicast (TG3_OPT_SCAN_PAIR; 300 rotations = 3 row tiles, so one pair
    holds a tile past the last row) and with 32-wide K blocks in 64-byte
    swizzled stages (TG3_OPT_SCAN_BK) against the default form on the same
    inputs.  The pair and K-block forms issue the same MMAs in the same
    order: the same log-likelihoods to the last bit.  A narrower tile changes
    the MMA shape, so its sums may round differently: log-likelihoods within
    1e-6 relative, weights within 1e-4."""
    rng = np.random.default_rng(43)
    st = small["st"]
    nImg, nR, nT = 30, 300, 9
    q = synth.haar_quaternions(rng, nR)
    mat = np.ascontiguousarray(O.rotmat(q).reshape(-1, 9))
    trans = synth.global_translations(1, 1.0)
    pR = rng.random(nR) + 0.5
    pT = rng.random(nT) + 0.5
    args = [dev(st.dat[:nImg].astype(np.complex64)), dev(st.ctf[:nImg].astype(np.float32)),
            dev(st.sigRcp[:nImg].astype(np.float32)), dev(mat), dev(trans), dev(pR), dev(pT)]

    def run(tile_n, pair, bk):
        ctx.set_option(tg3.OPT_SCAN_TILE_N, tile_n)
        ctx.set_option(tg3.OPT_SCAN_PAIR, pair)
        ctx.set_option(tg3.OPT_SCAN_BK, bk)
        o = dict(wC=torch.empty(nImg, dtype=torch.float64, device=DEV),
                 wR=torch.empty((nImg, nR), dtype=torch.float64, device=DEV),
                 wT=torch.empty((nImg, nT), dtype=torch.float64, device=DEV),
                 base=torch.empty(nImg, dtype=torch.float64, device=DEV),
                 dvp=torch.empty((nImg, nR, nT), dtype=torch.float32, device=DEV))
        ctx.global_scan(0, nImg, nR, nT, *args, o["wC"], o["wR"], o["wT"], o["base"], o["dvp"],
                        tg3.SCORE_BF16X3)
        ctx.sync()
        return {k: v.cpu().numpy() for k, v in o.items()}

    try:
        a, b = run(*form), run(0, 0, 64)
    finally:
        ctx.set_option(tg3.OPT_SCAN_TILE_N, 0)
        ctx.set_option(tg3.OPT_SCAN_PAIR, 0)
        ctx.set_option(tg3.OPT_SCAN_BK, 32)
    for k in ("dvp", "wC", "wR", "wT", "base"):
        if form[0] == 0:
            np.testing.assert_array_equal(a[k], b[k])
        else:
            np.testing.assert_allclose(a[k], b[k], rtol=1e-6 if k in ("dvp", "base") else 1e-4,
                                       atol=0)


def test_local_phase_k_block_forms(small, ctx):
    """The split-bf16 local phase's cross term with 32-wide K blocks in
    64-byte swizzled stages (TG3_OPT_LOCAL_BK 32, a choice of the uneven-batch
    autotuner) against the default 64-wide blocks: the same MMAs in the same
    order, so the same log-likelihoods and weights to the last bit."""
    nP, nR, nT = 3, 300, 100
    d = _local_inputs(small, nP, nR, nT, 11)
    res = {}
    try:
        for bk in (32, 64):
            ctx.set_option(tg3.OPT_LOCAL_BK, bk)
            o = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                     wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                     wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                     base=torch.empty(nP, dtype=torch.float64, device=DEV),
                     dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
            ctx.local_phase(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]),
                            dev(d["qs"]), dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]),
                            dev(d["pwC"]), None, o["wC"], o["wR"], o["wT"], o["base"], o["dvp"],
                            tg3.SCORE_BF16X3)
            ctx.sync()
            res[bk] = {k: v.cpu().numpy() for k, v in o.items()}
    finally:
        ctx.set_option(tg3.OPT_LOCAL_BK, 64)
    for k in ("dvp", "wC", "wR", "wT", "base"):
        np.testing.assert_array_equal(res[32][k], res[64][k])


@pytest.mark.parametrize("shape", [(4, 96, 21), (3, 300, 100), (2, 129, 7)])
def test_fused_matches_two_kernel_form(small, ctx, shape):
    """The fused projection + split-bf16 kernel (slices gathered straight into
    the tensor-core operand) against the two-kernel form (slice bank in HBM,
    then the GEMM) on the same inputs: likelihoods within 1e-5 relative."""
    nP, nR, nT = shape
    d = _local_inputs(small, nP, nR, nT, 5)
    res = {}
    for fused in (1, 0):
        ctx.set_option(tg3.OPT_FUSED, fused)
        o = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                 wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                 wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                 base=torch.empty(nP, dtype=torch.float64, device=DEV),
                 dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
        ctx.local_phase(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]), dev(d["qs"]),
                        dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]), dev(d["pwC"]), None,
                        o["wC"], o["wR"], o["wT"], o["base"], o["dvp"], tg3.SCORE_BF16X3)
        ctx.sync()
        res[fused] = {k: v.cpu().numpy() for k, v in o.items()}
    ctx.set_option(tg3.OPT_FUSED, 0)
    f, u = res[1], res[0]
    rel = np.abs(f["dvp"] - u["dvp"]) / np.abs(u["dvp"])
    assert rel.max() < 1e-5, rel.max()
    assert np.all(np.argmax(f["dvp"].reshape(nP, -1), 1) == np.argmax(u["dvp"].reshape(nP, -1), 1))
    assert np.allclose(f["base"], u["base"], rtol=1e-6)


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3])
def test_local_phase_from_bank(small, precision):
    """Rotations given as rows of a projection bank score as the same
    rotations projected directly (the bank rows are the same projections; the
    row norms are summed in another order)."""
    nP, nR, nT, nB = 4, 48, 21, 150
    rng = np.random.default_rng(61)
    d = _local_inputs(small, nP, nR, nT, 5)
    bq = synth.haar_quaternions(rng, nB)
    bq[:nP] = small["st"].quat_true[:nP]
    idx = rng.integers(0, nB, (nP, nR)).astype(np.int32)
    idx[:, 0] = np.arange(nP)                  # each particle's true pose among them
    c = tg3.Context(0)
    try:
        c.set_volume(0, torch.as_tensor(small["vol32"]).to(DEV), small["pf"])
        c.set_pixels(small["iCol"], small["iRow"], small["box"])
        c.set_bank(0, dev(bq), nB)
        res = []
        for use_bank in (True, False):
            o = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                     wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                     wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                     base=torch.empty(nP, dtype=torch.float64, device=DEV),
                     dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
            args = (dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]))
            rest = (dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]), dev(d["pwC"]), None,
                    o["wC"], o["wR"], o["wT"], o["base"], o["dvp"], precision)
            if use_bank:
                c.local_phase_bank(nP, nR, nT, *args, dev(idx), *rest)
            else:
                c.local_phase(nP, nR, nT, *args, dev(np.ascontiguousarray(bq[idx])), *rest)
            c.sync()
            res.append({k: v.cpu().numpy() for k, v in o.items()})
        a, b = res
        np.testing.assert_allclose(a["dvp"], b["dvp"], rtol=2e-5)
        np.testing.assert_allclose(a["base"], b["base"], rtol=1e-6)
        for k in ("wR", "wT"):
            np.testing.assert_allclose(a[k] / a[k].sum(1, keepdims=True),
                                       b[k] / b[k].sum(1, keepdims=True), atol=1e-4)
        assert np.array_equal(a["wR"].argmax(1), b["wR"].argmax(1))
        # an index outside the bank is reported, and the context stays usable
        bad = idx.copy()
        bad[1, 3] = nB
        o = res[0]
        outs = [torch.empty(x.shape, dtype=torch.float64 if x.dtype == np.float64 else
                            torch.float32, device=DEV) for x in (o["wC"], o["wR"], o["wT"],
                                                                  o["base"], o["dvp"])]
        c.local_phase_bank(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]), dev(bad),
                           dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]), dev(d["pwC"]), None,
                           *outs, precision)
        with pytest.raises(tg3.TG3Error):
            c.sync()
        c.sync()
        # a bank built on another pixel set is refused
        c.set_pixels(small["iCol"][:-5], small["iRow"][:-5], small["box"])
        with pytest.raises(tg3.TG3Error):
            c.local_phase_bank(nP, nR, nT, dev(d["dat"]), dev(d["ctf"]), dev(d["sig"]),
                               dev(idx), dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]),
                               dev(d["pwC"]), None, *outs, precision)
    finally:
        c.close()


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3])
def test_local_phase_defocus_search(small, precision):
    """The defocus search of Optimiser::updateSP (SEARCH_TYPE_CTF): every
    (rotation, translation, defocus) hypothesis scored with the CTF at the
    particle's defocus scaled by that hypothesis' factor.  The oracle scores
    each defocus with score_local and merges the results to the particle's
    best hypothesis, as the running baseline does."""
    nP, nR, nT, nD = 3, 40, 9, 3
    d = _local_inputs(small, nP, nR, nT, 9)
    rng = np.random.default_rng(67)
    attr = synth.ctf_attrs(rng, nP)
    factors = np.array([[0.96, 1.0, 1.04], [0.9, 1.0, 1.1], [1.0, 1.02, 0.98]])
    ctfD = np.empty((nP, nD, d["K"]), np.float32)
    for k in range(nD):
        a = attr.copy()
        a[:, 1] *= factors[:, k]
        a[:, 2] *= factors[:, k]
        ctfD[:, k] = synth.ctf_values(a, small["px"], small["box"], small["iCol"],
                                      small["iRow"]).astype(np.float32)
    pwD = rng.random((nP, nD)) + 0.5
    c = tg3.Context(0)
    try:
        c.set_volume(0, torch.as_tensor(small["vol32"]).to(DEV), small["pf"])
        c.set_pixels(small["iCol"], small["iRow"], small["box"])
        o = dict(wC=torch.empty(nP, dtype=torch.float64, device=DEV),
                 wR=torch.empty((nP, nR), dtype=torch.float64, device=DEV),
                 wT=torch.empty((nP, nT), dtype=torch.float64, device=DEV),
                 wD=torch.empty((nP, nD), dtype=torch.float64, device=DEV),
                 base=torch.empty(nP, dtype=torch.float64, device=DEV),
                 dvp=torch.empty((nP, nD, nR, nT), dtype=torch.float32, device=DEV))
        c.local_phase_ctf(nP, nR, nT, nD, dev(d["dat"]), dev(ctfD), dev(d["sig"]), dev(d["qs"]),
                          dev(d["ts"]), dev(d["pwR"]), dev(d["pwT"]), dev(pwD), dev(d["pwC"]),
                          None, o["wC"], o["wR"], o["wT"], o["wD"], o["base"], o["dvp"],
                          precision)
        c.sync()
        g = {k: v.cpu().numpy() for k, v in o.items()}
    finally:
        c.close()
    for l in range(nP):
        rs = [O.score_local(small["vol"], small["pf"], small["iCol"], small["iRow"], small["box"],
                            f32(d["dat"][l]), f32(ctfD[l, k]), f32(d["sig"][l]), f32(d["qs"][l]),
                            f32(d["ts"][l]), d["pwR"][l], d["pwT"][l], 1.0) for k in range(nD)]
        for k in range(nD):
            rel = np.abs(g["dvp"][l, k] - rs[k]["dvp"]) / np.abs(rs[k]["dvp"])
            assert rel.max() < 1e-4, (k, rel.max())
        base = max(r["base"] for r in rs)
        assert abs(g["base"][l] - base) / abs(base) < 1e-4
        e = np.array([np.exp(r["base"] - base) for r in rs])
        wD = e * np.array([r["wC"] for r in rs])
        wR = sum(pwD[l, k] * e[k] * rs[k]["wR"] for k in range(nD))
        wT = sum(pwD[l, k] * e[k] * rs[k]["wT"] for k in range(nD))
        for got, ref in ((g["wD"][l], wD), (g["wR"][l], wR), (g["wT"][l], wT)):
            assert np.abs(got / got.sum() - ref / ref.sum()).max() < 2e-3
        assert np.argmax(g["wD"][l]) == np.argmax(wD)


def test_expect_local3d_defocus_host(small):
    """The reference-shaped defocus search (ExpectLocalP / RTD / PreI3D / M
    with k1 != 0): CTFs made on the device from the per-pixel defocus and
    frequency (kernel_CalCTFL's formula) for each defocus factor."""
    st = small["st"]
    nR, nT, nD = 48, 9, 3
    d = _local_inputs(small, 1, nR, nT, 37)
    rng = np.random.default_rng(71)
    attr = synth.ctf_attrs(rng, 1)[0]
    V, dU, dV, th, Cs, A, ps = attr
    lam = 12.2643247 / np.sqrt(V * (1 + V * 0.978466e-6))
    k1, k2 = np.pi * lam, (np.pi / 2) * Cs * lam ** 3
    iCol, iRow = small["iCol"], small["iRow"]
    freq = np.hypot(iCol, iRow) / (small["px"] * small["box"])
    ang = np.arctan2(iRow, iCol) - th
    defO = -(dU + dV + (dU - dV) * np.cos(2 * ang)) / 2
    dpara = np.array([0.95, 1.0, 1.05])
    pwD = np.array([0.2, 0.5, 0.3])
    vol = np.ascontiguousarray(small["vol32"])
    h = tg3.ctypes.c_void_p()
    tg3.check(tg3.lib().tg3_volume_create(tg3.ctypes.byref(h), tg3.ptr(vol), vol.shape[0],
                                          small["pf"]))
    try:
        wC = np.zeros(1, np.float32)
        wR = np.zeros(nR, np.float32)
        wT = np.zeros(nT, np.float32)
        wD = np.zeros(nD, np.float32)
        dvp = np.zeros((nD, nR, nT), np.float32)
        bl = np.zeros(1, np.float32)
        # every array the call reads is held here: a temporary passed by
        # address would be freed before the call
        c = lambda x, dt: np.ascontiguousarray(x, dtype=dt)
        q, t = c(d["qs"][0], np.float64), c(d["ts"][0], np.float64)
        dat, sig = c(d["dat"][0], np.complex64), c(d["sig"][0], np.float32)
        dO, fq = c(defO, np.float32), c(freq, np.float32)
        ic, ir = c(iCol, np.int32), c(iRow, np.int32)
        dp, pr, pt, pd = (c(dpara, np.float64), c(d["pwR"][0], np.float64),
                          c(d["pwT"][0], np.float64), c(pwD, np.float64))
        tg3.check(tg3.lib().tg3_ExpectLocal3D_ctf(
            h, tg3.ptr(dat), tg3.ptr(dO), tg3.ptr(fq), k1, k2, ps, A, tg3.ptr(sig), tg3.ptr(ic),
            tg3.ptr(ir), st.K, small["box"], tg3.ptr(q), nR, tg3.ptr(t), nT, tg3.ptr(dp), nD,
            tg3.ptr(pr), tg3.ptr(pt), tg3.ptr(pd), 1.0, tg3.ptr(wC), tg3.ptr(wR), tg3.ptr(wT),
            tg3.ptr(wD), tg3.ptr(dvp), tg3.ptr(bl)))
    finally:
        tg3.lib().tg3_volume_destroy(h)
    rs = []
    for k in range(nD):
        a = attr.copy()
        a[1] *= dpara[k]
        a[2] *= dpara[k]
        ctf_k = synth.ctf_values(a[None], small["px"], small["box"], iCol, iRow)[0]
        rs.append(O.score_local(small["vol"], small["pf"], iCol, iRow, small["box"],
                                f32(d["dat"][0]), f32(ctf_k), f32(d["sig"][0]), f32(q), f32(t),
                                d["pwR"][0], d["pwT"][0], 1.0))
    for k in range(nD):
        assert (np.abs(dvp[k] - rs[k]["dvp"]) / np.abs(rs[k]["dvp"])).max() < 1e-4
    base = max(r["base"] for r in rs)
    e = np.array([np.exp(r["base"] - base) for r in rs])
    wD_ref = e * np.array([r["wC"] for r in rs])
    wR_ref = sum(pwD[k] * e[k] * rs[k]["wR"] for k in range(nD))
    np.testing.assert_allclose(wD / wD.sum(), wD_ref / wD_ref.sum(), atol=2e-3)
    np.testing.assert_allclose(wR / wR.sum(), wR_ref / wR_ref.sum(), atol=2e-3)


@pytest.mark.parametrize("kernel", [tg3.KERNEL_MKB, tg3.KERNEL_TRILINEAR])
def test_insertft_defocus_host(small, kernel):
    """InsertFT with the defocus search: every draw's CTF from its image's
    attributes with the draw's defocus factor (kernel_CalculateCTF); ctfP
    is not read."""
    rng = np.random.default_rng(73)
    st = small["st"]
    K, pf, box = st.K, small["pf"], small["box"]
    vdim = pf * box
    nImg, mReco = 4, 3
    quats = synth.haar_quaternions(rng, nImg * mReco)
    trans = rng.uniform(-2, 2, (nImg * mReco, 2))
    offS = rng.uniform(-0.5, 0.5, (nImg, 2))
    w = (np.ones(nImg) / mReco).astype(np.float32)
    attr = synth.ctf_attrs(rng, nImg)
    attr32 = np.ascontiguousarray(attr.astype(np.float32))
    nD = rng.uniform(0.9, 1.1, nImg * mReco)
    F = np.zeros((vdim, vdim, vdim // 2 + 1), np.complex64)
    T = np.zeros((vdim, vdim, vdim // 2 + 1), np.float32)
    O3D = np.zeros(3)
    counter = np.zeros(1, np.int32)
    dat = np.ascontiguousarray(st.dat[:nImg].astype(np.complex64))
    sig = np.ascontiguousarray(st.sigRcp[:nImg].astype(np.float32))
    iColPad = np.ascontiguousarray(small["iCol"] * pf, np.int32)
    iRowPad = np.ascontiguousarray(small["iRow"] * pf, np.int32)
    tg3.check(tg3.lib().tg3_InsertFT(
        tg3.ptr(F), tg3.ptr(T), tg3.ptr(O3D), tg3.ptr(counter), tg3.ptr(dat), None,
        tg3.ptr(sig), tg3.ptr(attr32), tg3.ptr(offS), tg3.ptr(w), tg3.ptr(quats), tg3.ptr(trans),
        tg3.ptr(nD), tg3.ptr(iColPad), tg3.ptr(iRowPad),
        small["px"], 1, pf, K, mReco, box, vdim, nImg, kernel))
    assert counter[0] == nImg * mReco
    Fr = np.zeros(F.shape, np.complex128)
    Tr = np.zeros(T.shape)
    b = (pf * 1.9) ** 2
    tab = O.mkb_table(1.9, 15.0, b, 100000)
    mats = O.rotmat(quats)
    for l in range(nImg):
        for m in range(mReco):
            d = l * mReco + m
            a = attr32[l].astype(np.float64)
            a[1] *= nD[d]
            a[2] *= nD[d]
            ctf_d = synth.ctf_values(a[None], small["px"], box, small["iCol"], small["iRow"])[0]
            tt = f32(trans[d]) - f32(offS[l])
            img = O.translate_image(f32(dat[l]), -tt[0], -tt[1], box, small["iCol"], small["iRow"])
            O.insert(Fr, Tr, img, f32(ctf_d), mats[d], float(w[l]), small["iCol"] * pf,
                     small["iRow"] * pf, kernel, pf * 1.9, tab, b)
    assert np.abs(F - Fr).max() < 2e-4 * np.abs(Fr).max()
    assert np.abs(T - Tr).max() < 2e-4 * np.abs(Tr).max()


def test_expect_global2d_host():
    """2-D classification's global search (ExpectGlobal2D) against the
    oracle: the 2-D projection of every class (or_project2d, pinned to the
    reference's Image::getByInterpolationFT) scored by the multi-class global
    scan with its running baseline over classes."""
    rng = np.random.default_rng(83)
    box, pf, px = 24, 2, 1.5
    vdim = box * pf
    iCol, iRow = synth.pixel_index(box, 10, synth.config_rL(box, px))[:2]
    K = len(iCol)
    nK, nR, nImg = 2, 36, 6
    imgs = (rng.standard_normal((nK, vdim, vdim // 2 + 1)) +
            1j * rng.standard_normal((nK, vdim, vdim // 2 + 1))).astype(np.complex64)
    ang = np.arange(nR) * (2 * np.pi / nR)
    rot = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    trans = np.ascontiguousarray(synth.global_translations(1, 1.0))
    nT = len(trans)
    attr = synth.ctf_attrs(rng, nImg)
    ctf = np.ascontiguousarray(synth.ctf_values(attr, px, box, iCol, iRow).astype(np.float32))
    sig = np.full((nImg, K), -0.5, np.float32)
    traP = O.translate(trans, box, iCol, iRow)
    rotP = [O.project2d(imgs[k].astype(np.complex128), rot, iCol, iRow, pf) for k in range(nK)]
    kt, rt, tt = rng.integers(0, nK, nImg), rng.integers(0, nR, nImg), rng.integers(0, nT, nImg)
    dat = np.stack([ctf[l] * rotP[kt[l]][rt[l]] * traP[tt[l]] for l in range(nImg)])
    dat = np.ascontiguousarray((dat + 0.3 * (rng.standard_normal(dat.shape) +
                                             1j * rng.standard_normal(dat.shape))).astype(np.complex64))
    pR = np.full(nR, 1.0 / nR)
    pT = np.full(nT, 1.0 / nT)
    wC = np.zeros(nImg * nK, np.float32)
    wR = np.zeros(nImg * nK * nR, np.float32)
    wT = np.zeros(nImg * nK * nT, np.float32)
    vol = np.ascontiguousarray(imgs)
    ic, ir = np.ascontiguousarray(iCol, np.int32), np.ascontiguousarray(iRow, np.int32)
    tg3.check(tg3.lib().tg3_ExpectGlobal2D(
        tg3.ptr(vol), tg3.ptr(dat), tg3.ptr(ctf), tg3.ptr(sig), tg3.ptr(trans), tg3.ptr(wC),
        tg3.ptr(wR), tg3.ptr(wT), tg3.ptr(pR), tg3.ptr(pT), tg3.ptr(rot), tg3.ptr(ic),
        tg3.ptr(ir), nK, nR, nT, pf, 1, box, vdim, K, nImg))
    state = None
    for k in range(nK):
        res = O.score_global(rotP[k], traP, f32(dat), f32(ctf), f32(sig), pR, pT, kIdx=k, nK=nK,
                             state=state, want_dvp=False)
        state = (res["wC"], res["wR"], res["wT"], res["baseL"])
    rC, rR = state[0].reshape(nImg, nK), state[1].reshape(nImg, nK, nR)
    gC, gR = wC.reshape(nImg, nK), wR.reshape(nImg, nK, nR)
    np.testing.assert_allclose(gC / gC.sum(1, keepdims=True), rC / rC.sum(1, keepdims=True),
                               atol=2e-3)
    for l in range(nImg):
        k = int(np.argmax(rC[l]))
        assert int(np.argmax(gC[l])) == k == kt[l]
        assert int(np.argmax(gR[l, k])) == int(np.argmax(rR[l, k])) == rt[l]
        np.testing.assert_allclose(gR[l, k] / gR[l, k].sum(), rR[l, k] / rR[l, k].sum(),
                                   atol=2e-3)


def test_global_scan2d_device_split(small):
    """The device 2-D scan in both precisions gives the same best rotation and
    log-likelihoods within the split path's bound."""
    rng = np.random.default_rng(89)
    box, pf = small["box"], small["pf"]
    vdim = box * pf
    img = (rng.standard_normal((vdim, vdim // 2 + 1)) +
           1j * rng.standard_normal((vdim, vdim // 2 + 1))).astype(np.complex64)
    nR, nImg = 24, 4
    ang = rng.uniform(0, 2 * np.pi, nR)
    rot = np.stack([np.cos(ang), np.sin(ang)], 1)
    trans = synth.global_translations(1, 1.0)
    nT = len(trans)
    st = small["st"]
    out = {}
    c = tg3.Context(0)
    try:
        c.set_pixels(small["iCol"], small["iRow"], box)
        # device inputs held here: a temporary passed by address would be freed
        ins = [dev(x) for x in (img, st.dat[:nImg].astype(np.complex64),
                                st.ctf[:nImg].astype(np.float32),
                                st.sigRcp[:nImg].astype(np.float32), rot, trans,
                                np.full(nR, 1.0 / nR), np.full(nT, 1.0 / nT))]
        for prec in (tg3.SCORE_FP32, tg3.SCORE_BF16X3):
            o = [torch.empty(s, dtype=torch.float64, device=DEV)
                 for s in (nImg, (nImg, nR), (nImg, nT), nImg)]
            dvp = torch.empty((nImg, nR, nT), dtype=torch.float32, device=DEV)
            tg3.check(tg3.lib().tg3_global_scan2d_d(
                c.h, tg3.ptr(ins[0]), vdim, pf, nImg, nR, nT, tg3.ptr(ins[1]), tg3.ptr(ins[2]),
                tg3.ptr(ins[3]), tg3.ptr(ins[4]), tg3.ptr(ins[5]), tg3.ptr(ins[6]),
                tg3.ptr(ins[7]), tg3.ptr(o[0]), tg3.ptr(o[1]), tg3.ptr(o[2]), tg3.ptr(o[3]),
                tg3.ptr(dvp), prec))
            c.sync()
            out[prec] = dvp.cpu().numpy()
    finally:
        c.close()
    a, b = out[tg3.SCORE_FP32], out[tg3.SCORE_BF16X3]
    assert np.abs(a - b).max() / np.abs(a).max() < 1e-4
    assert np.array_equal(a.reshape(nImg, -1).argmax(1), b.reshape(nImg, -1).argmax(1))


@pytest.mark.parametrize("csearch", [0, 1])
def test_insert_i2d_host(csearch):
    """2-D classification's insertion (InsertI2D) against the oracle: each
    draw's shifted image, times its CTF and its image's weight, added
    bilinearly at the draw's in-plane rotation into its class (or_insert2d,
    pinned to the reference's Image::addFT); O2D and counter per class.
    With the defocus search every draw's CTF comes from its image's
    attributes and the draw's defocus factor."""
    rng = np.random.default_rng(97)
    box, pf, px = 24, 2, 1.5
    vdim = box * pf
    nx = vdim // 2 + 1
    iCol, iRow = synth.pixel_index(box, 10, synth.config_rL(box, px))[:2]
    K = len(iCol)
    nK, nImg, mReco = 3, 7, 2
    nd = nImg * mReco
    dat = np.ascontiguousarray((rng.standard_normal((nImg, K)) +
                                1j * rng.standard_normal((nImg, K))).astype(np.complex64))
    attr = synth.ctf_attrs(rng, nImg)
    attr32 = np.ascontiguousarray(attr.astype(np.float32))
    ctf = np.ascontiguousarray(synth.ctf_values(attr, px, box, iCol, iRow).astype(np.float32))
    sig = np.full((nImg, K), 1.0, np.float32)
    w = rng.uniform(0.2, 1.0, nImg).astype(np.float32)
    offS = rng.uniform(-0.5, 0.5, (nImg, 2))
    nC = np.ascontiguousarray(rng.integers(0, nK, nd), np.int32)
    ang = rng.uniform(0, 2 * np.pi, nd)
    nR = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    nT = rng.uniform(-2, 2, (nd, 2))
    nD = rng.uniform(0.9, 1.1, nd)
    F = np.zeros((nK, vdim, nx), np.complex64)
    F[1, 2, 3] = 1 - 1j       # accumulated into, not overwritten
    T = np.zeros((nK, vdim, nx), np.float32)
    O2D = np.zeros((nK, 2))
    O2D[0] = (0.5, -0.25)
    counter = np.zeros(nK, np.int32)
    counter[2] = 4
    iColPad = np.ascontiguousarray(iCol * pf, np.int32)
    iRowPad = np.ascontiguousarray(iRow * pf, np.int32)
    tg3.check(tg3.lib().tg3_InsertI2D(
        tg3.ptr(F), tg3.ptr(T), tg3.ptr(O2D), tg3.ptr(counter), tg3.ptr(dat),
        None if csearch else tg3.ptr(ctf), tg3.ptr(sig), tg3.ptr(w), tg3.ptr(offS), tg3.ptr(nC),
        tg3.ptr(nR), tg3.ptr(nT), tg3.ptr(nD) if csearch else None,
        tg3.ptr(attr32) if csearch else None, tg3.ptr(iColPad), tg3.ptr(iRowPad), px, csearch,
        nK, pf, K, mReco, box, vdim, nImg))
    Fr = np.zeros(F.shape, np.complex128)
    Fr[1, 2, 3] = 1 - 1j
    Tr = np.zeros(T.shape)
    Or = np.array([[0.5, -0.25], [0, 0], [0, 0]])
    cr = np.array([0, 0, 4])
    for l in range(nImg):
        for m in range(mReco):
            d = l * mReco + m
            if csearch:
                a = attr32[l].astype(np.float64)
                a[1] *= nD[d]
                a[2] *= nD[d]
                c = synth.ctf_values(a[None], px, box, iCol, iRow)[0]
            else:
                c = ctf[l]
            tt = nT[d] - offS[l]
            img = O.translate_image(f32(dat[l]), -tt[0], -tt[1], box, iCol, iRow)
            k = nC[d]
            O.insert2d(Fr[k], Tr[k], img, f32(c), nR[d], float(w[l]), iColPad, iRowPad)
            c_, s_ = nR[d]
            Or[k] -= (c_ * tt[0] - s_ * tt[1], s_ * tt[0] + c_ * tt[1])
            cr[k] += 1
    np.testing.assert_array_equal(counter, cr)
    np.testing.assert_allclose(O2D, Or, rtol=0, atol=1e-9)
    assert np.abs(F - Fr).max() < 2e-4 * np.abs(Fr).max()
    assert np.abs(T - Tr).max() < 2e-4 * np.abs(Tr).max()


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_global_scan2d_classes_device(precision):
    """The multi-class device scan (every class's rotations as rows of one
    projection matrix, one cross-term GEMM) against the oracle's class-by-class
    scan with the running baseline: merged class weights and, for the best
    class, its rotation weights; the best class and rotation exactly."""
    rng = np.random.default_rng(101)
    box, pf, px = 24, 2, 1.5
    vdim = box * pf
    iCol, iRow = synth.pixel_index(box, 10, synth.config_rL(box, px))[:2]
    K = len(iCol)
    nK, nR, nImg = 5, 36, 9
    imgs = (rng.standard_normal((nK, vdim, vdim // 2 + 1)) +
            1j * rng.standard_normal((nK, vdim, vdim // 2 + 1))).astype(np.complex64)
    ang = np.arange(nR) * (2 * np.pi / nR)
    rot = np.ascontiguousarray(np.stack([np.cos(ang), np.sin(ang)], 1))
    trans = np.ascontiguousarray(synth.global_translations(1, 1.0))
    nT = len(trans)
    attr = synth.ctf_attrs(rng, nImg)
    ctf = np.ascontiguousarray(synth.ctf_values(attr, px, box, iCol, iRow).astype(np.float32))
    sig = np.full((nImg, K), -0.5, np.float32)
    traP = O.translate(trans, box, iCol, iRow)
    rotP = [O.project2d(imgs[k].astype(np.complex128), rot, iCol, iRow, pf) for k in range(nK)]
    kt, rt, tt = rng.integers(0, nK, nImg), rng.integers(0, nR, nImg), rng.integers(0, nT, nImg)
    dat = np.stack([ctf[l] * rotP[kt[l]][rt[l]] * traP[tt[l]] for l in range(nImg)])
    dat = np.ascontiguousarray((dat + 0.3 * (rng.standard_normal(dat.shape) +
                                             1j * rng.standard_normal(dat.shape))).astype(np.complex64))
    pR = np.full(nR, 1.0 / nR)
    pT = np.full(nT, 1.0 / nT)
    dev = "cuda:0"
    td = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(dev)
    wC = torch.empty((nImg, nK), dtype=torch.float32, device=dev)
    wR = torch.empty((nImg, nK, nR), dtype=torch.float32, device=dev)
    wT = torch.empty((nImg, nK, nT), dtype=torch.float32, device=dev)
    base = torch.empty(nImg, dtype=torch.float32, device=dev)
    ctx = tg3.Context(0)
    try:
        ctx.set_pixels(iCol, iRow, box)
        prec = tg3.SCORE_BF16X3 if precision == "bf16x3" else tg3.SCORE_FP32
        ctx.global_scan2d_classes(td(imgs), pf, nImg, nR, nT, td(dat), td(ctf), td(sig), td(rot),
                                  td(trans), td(pR), td(pT), wC, wR, wT, base, prec)
        ctx.sync()
    finally:
        ctx.close()
    state = None
    for k in range(nK):
        res = O.score_global(rotP[k], traP, f32(dat), f32(ctf), f32(sig), pR, pT, kIdx=k, nK=nK,
                             state=state, want_dvp=False)
        state = (res["wC"], res["wR"], res["wT"], res["baseL"])
    rC, rR = state[0].reshape(nImg, nK), state[1].reshape(nImg, nK, nR)
    gC, gR = wC.cpu().numpy(), wR.cpu().numpy()
    np.testing.assert_allclose(base.cpu().numpy(), state[3], rtol=1e-3)
    np.testing.assert_allclose(gC / gC.sum(1, keepdims=True), rC / rC.sum(1, keepdims=True),
                               atol=2e-3)
    for l in range(nImg):
        k = int(np.argmax(rC[l]))
        assert int(np.argmax(gC[l])) == k == kt[l]
        assert int(np.argmax(gR[l, k])) == int(np.argmax(rR[l, k])) == rt[l]
        np.testing.assert_allclose(gR[l, k] / gR[l, k].sum(), rR[l, k] / rR[l, k].sum(),
                                   atol=2e-3)
