"""The learned E-step entry points (tg3_learned_expect_d and its host-buffer
form tg3_ExpectLearned3D) against the library's separate calls and the
oracle.

The entry chains the network, the matching proposals, the exact rescoring
from the projection banks, the proposal confidence and the global-search
fallback.  Each link is checked here on a small box-128 case with three
classes and an untrained network (the chain does not depend on what the
network has learned):
- the proposals equal tg3_cnn_match_propose per class;
- the rescoring equals tg3_local_phase_bank_d on the same proposals, and its
  log-likelihoods equal the oracle's within the FP32 bar (1e-4 relative);
- the confidence equals (max - median) / (1.4826 (MAD + 1e-12)) computed here;
- with every particle falling back, the poses and best log-likelihoods
  equal the global search over the bank's rotations (tg3_global_scan_d);
- the host-buffer form returns what the device form returns."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
import tg3
from tg3 import learned, synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
F64 = dict(dtype=torch.float64, device=DEV)


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(91)
    box, px, pf, rU = 128, 1.4, 2, 32
    maps = [synth.blob_map(rng, 60, (1.5, 3.0), px, 40.0) for _ in range(3)]
    rL = synth.config_rL(box, px)
    iCol, iRow, _, _ = synth.pixel_index(box, rU, rL)
    nv = synth.signal_power(maps, box, px, rU, rL, device=DEV) / 0.5 / 2.0
    ps = synth.particle_set_dev(92, maps, np.array([0, 1, 2, 2, 1, 0, 0, 2, 1, 1, 0, 2]), box, px,
                                rU, rL, 2.0, nv, device=DEV)
    ctx = tg3.Context(0)
    net = tg3.Cnn(0, seed=93)
    vols = []
    for c, bm in enumerate(maps):
        v = synth.padded_volume(bm, box, pf, device=DEV, dtype=torch.float32)
        vols.append(v)
        ctx.set_volume(c, v, pf)
    qg = synth.global_rotations(2, 12)                  # 48 directions x 12 angles = 576
    emb = {c: learned.reference_embeddings(net, learned.render_references(ctx, c, qg, box))
           for c in range(3)}
    ctx.set_pixels(iCol, iRow, box)
    qg_d = torch.as_tensor(qg, **F64)
    for c in range(3):
        ctx.set_bank(c, qg_d, len(qg))
        ctx.set_references(c, emb[c])
    gt = torch.as_tensor(synth.global_translations(2, 1.0), **F64)     # 5 x 5
    yield dict(ctx=ctx, net=net, ps=ps, qg=qg, qg_d=qg_d, emb=emb, gt=gt, box=box, pf=pf,
               vols=vols, cls=torch.as_tensor(ps.cls.astype(np.int32), device=DEV))
    net.close()
    ctx.close()


def _outputs(n, nR, nT):
    return dict(bestQuat=torch.empty((n, 4), **F64), bestTrans=torch.empty((n, 2), **F64),
                baseL=torch.empty(n, **F64),
                peak=torch.empty(n, dtype=torch.float32, device=DEV),
                fellBack=torch.empty(n, dtype=torch.int32, device=DEV),
                propIdx=torch.empty((n, nR), dtype=torch.int32, device=DEV),
                propQuat=torch.empty((n, nR, 4), **F64),
                propTrans=torch.empty((n, nT, 2), **F64),
                propWR=torch.empty((n, nR), **F64), propWT=torch.empty((n, nT), **F64),
                propBase=torch.empty(n, **F64),
                propDvp=torch.empty((n, nR, nT), dtype=torch.float32, device=DEV))


def _run(c, peak_min, precision, nR=32, nT=9, seed=5):
    ps = c["ps"]
    o = _outputs(len(ps.cls), nR, nT)
    c["ctx"].learned_expect(c["net"], ps.images, ps.dat, ps.ctf, ps.sigRcp, c["cls"], nR, nT,
                            seed, c["gt"], peak_min, precision, o)
    return {k: v.cpu().numpy() for k, v in o.items()}


def test_proposals_rescoring_and_confidence(case):
    nR, nT = 32, 9
    r = _run(case, float("-inf"), tg3.SCORE_FP32, nR, nT)
    ps, ctx, n = case["ps"], case["ctx"], len(case["ps"].cls)
    assert not r["fellBack"].any()
    # proposals: the class-by-class matching of the same network outputs
    out = torch.empty((n, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    case["net"].infer(ps.images, out)
    for c in range(3):
        sel = np.nonzero(ps.cls == c)[0]
        q = torch.empty((len(sel), nR, 4), **F64)
        t = torch.empty((len(sel), nT, 2), **F64)
        ix = torch.empty((len(sel), nR), dtype=torch.int32, device=DEV)
        tg3.Cnn.match_propose(out[torch.as_tensor(sel, device=DEV)].contiguous(), case["emb"][c],
                              case["qg_d"], nR, nT, 5, q, t, ix)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(ix.cpu().numpy(), r["propIdx"][sel])
        np.testing.assert_array_equal(q.cpu().numpy(), r["propQuat"][sel])
    # rescoring: the bank-row local phase on the entry's own proposals
    o = dict(wC=torch.empty(n, **F64), wR=torch.empty((n, nR), **F64),
             wT=torch.empty((n, nT), **F64), base=torch.empty(n, **F64),
             dvp=torch.empty((n, nR, nT), dtype=torch.float32, device=DEV))
    ctx.local_phase_bank(n, nR, nT, ps.dat, ps.ctf, ps.sigRcp,
                         torch.as_tensor(r["propIdx"], device=DEV),
                         torch.as_tensor(r["propTrans"], **F64),
                         torch.full((n, nR), 1.0 / nR, **F64), torch.full((n, nT), 1.0 / nT, **F64),
                         torch.ones(n, **F64), case["cls"], o["wC"], o["wR"], o["wT"], o["base"],
                         o["dvp"], tg3.SCORE_FP32)
    ctx.sync()
    np.testing.assert_array_equal(o["dvp"].cpu().numpy(), r["propDvp"])
    np.testing.assert_array_equal(o["base"].cpu().numpy(), r["propBase"])
    # best pose: argmax of the marginals
    ar = np.arange(n)
    np.testing.assert_array_equal(r["bestQuat"], r["propQuat"][ar, r["propWR"].argmax(1)])
    np.testing.assert_array_equal(r["bestTrans"], r["propTrans"][ar, r["propWT"].argmax(1)])
    np.testing.assert_array_equal(r["baseL"], r["propBase"])
    # confidence
    d = r["propDvp"].reshape(n, -1).astype(np.float64)
    med = np.median(d, 1)
    mad = np.median(np.abs(d - med[:, None]), 1) + 1e-12
    np.testing.assert_allclose(r["peak"], (d.max(1) - med) / (1.4826 * mad), rtol=1e-4)
    # the rescored log-likelihoods against the oracle (FP32 bar)
    for l in (0, 1, 3):
        c = int(ps.cls[l])
        vol = case["vols"][c].cpu().numpy().astype(np.complex128)
        ref = O.score_local(vol, case["pf"], ps.iCol, ps.iRow, case["box"],
                            ps.dat[l].cpu().numpy().astype(np.complex128),
                            ps.ctf[l].cpu().numpy().astype(np.float64),
                            ps.sigRcp[l].cpu().numpy().astype(np.float64), r["propQuat"][l],
                            r["propTrans"][l], np.full(nR, 1.0 / nR), np.full(nT, 1.0 / nT))
        rel = np.abs(r["propDvp"][l] - ref["dvp"]) / np.abs(ref["dvp"])
        assert rel.max() < 1e-4, rel.max()
        assert np.argmax(r["propDvp"][l]) == np.argmax(ref["dvp"])


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3])
def test_fallback_is_the_global_search(case, precision):
    r = _run(case, float("inf"), precision)
    ps, ctx, n = case["ps"], case["ctx"], len(case["ps"].cls)
    assert r["fellBack"].all()
    qg, gt = case["qg"], case["gt"]
    nRg, nTg = len(qg), gt.shape[0]
    # the rotation matrices made on the device from the same quaternions, as
    # the bank's projections were
    mats = torch.empty((nRg, 9), **F64)
    tg3.check(tg3.lib().tg3_rotmat_d(tg3.ptr(case["qg_d"]), nRg, tg3.ptr(mats), None))
    torch.cuda.synchronize()
    for c in range(3):
        sel = np.nonzero(ps.cls == c)[0]
        idx = torch.as_tensor(sel, device=DEV)
        m = len(sel)
        o = dict(wC=torch.empty(m, **F64), wR=torch.empty((m, nRg), **F64),
                 wT=torch.empty((m, nTg), **F64), base=torch.empty(m, **F64))
        ctx.global_scan(c, m, nRg, nTg, ps.dat[idx].contiguous(), ps.ctf[idx].contiguous(),
                        ps.sigRcp[idx].contiguous(), mats, gt, torch.full((nRg,), 1.0 / nRg, **F64),
                        torch.full((nTg,), 1.0 / nTg, **F64), o["wC"], o["wR"], o["wT"],
                        o["base"], None, precision)
        ctx.sync()
        np.testing.assert_array_equal(r["bestQuat"][sel], qg[o["wR"].argmax(1).cpu().numpy()])
        np.testing.assert_array_equal(r["bestTrans"][sel],
                                      gt.cpu().numpy()[o["wT"].argmax(1).cpu().numpy()])
        np.testing.assert_allclose(r["baseL"][sel], o["base"].cpu().numpy(), rtol=1e-6)


def test_host_form_matches_device_form(case):
    ps, n = case["ps"], len(case["ps"].cls)
    r0 = _run(case, float("-inf"), tg3.SCORE_BF16X3)
    tau = float(np.median(r0["peak"]))        # about half the particles fall back
    r = _run(case, tau, tg3.SCORE_BF16X3)
    assert 0 < r["fellBack"].sum() < n
    h = dict(q=np.zeros((n, 4)), t=np.zeros((n, 2)), b=np.zeros(n),
             pk=np.zeros(n, np.float32), fb=np.zeros(n, np.int32))
    case["ctx"].learned_expect_host(case["net"], ps.images.cpu().numpy(), ps.dat.cpu().numpy(),
                                    ps.ctf.cpu().numpy(), ps.sigRcp.cpu().numpy(),
                                    ps.cls.astype(np.int32), 32, 9, 5, case["gt"].cpu().numpy(),
                                    tau, tg3.SCORE_BF16X3, h["q"], h["t"], h["b"], h["pk"],
                                    h["fb"])
    np.testing.assert_array_equal(h["q"], r["bestQuat"])
    np.testing.assert_array_equal(h["t"], r["bestTrans"])
    np.testing.assert_array_equal(h["b"], r["baseL"])
    np.testing.assert_array_equal(h["fb"], r["fellBack"])


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("form", [0, 2])
@pytest.mark.parametrize("nR", [32, 160])
def test_bank_rows_straight_into_the_cross_term(case, nR, form, order):
    """The split-bf16 bank-row local phase with the operand tiles loaded
    straight from the banks (norms from the staged tiles) against the form
    that first copies the rows out (TG3_OPT_BANK_GATHER 1; form 0 gathers
    the tiles with the warps' own cp.async copies, form 2 with TMA gathers),
    with the particles visited in their own order and sorted by first
    proposed row (TG3_OPT_BANK_ORDER), and against the oracle:
    log-likelihoods within 1e-4 relative, the same best hypothesis,
    marginals within 2e-3 as distributions.  nR = 160 leaves a partial
    second row tile."""
    ps, ctx, n = case["ps"], case["ctx"], len(case["ps"].cls)
    nT = 9
    rng = np.random.default_rng(nR)
    idx = torch.as_tensor(rng.integers(0, len(case["qg"]), (n, nR)).astype(np.int32), device=DEV)
    trans = torch.as_tensor(rng.uniform(-2, 2, (n, nT, 2)), **F64)

    def run(opt):
        ctx.set_option(tg3.OPT_BANK_GATHER, int(opt))
        o = dict(wC=torch.empty(n, **F64), wR=torch.empty((n, nR), **F64),
                 wT=torch.empty((n, nT), **F64), base=torch.empty(n, **F64),
                 dvp=torch.empty((n, nR, nT), dtype=torch.float32, device=DEV))
        ctx.local_phase_bank(n, nR, nT, ps.dat, ps.ctf, ps.sigRcp, idx, trans,
                             torch.full((n, nR), 1.0 / nR, **F64),
                             torch.full((n, nT), 1.0 / nT, **F64), torch.ones(n, **F64),
                             case["cls"], o["wC"], o["wR"], o["wT"], o["base"], o["dvp"],
                             tg3.SCORE_BF16X3)
        ctx.sync()
        return {k: v.cpu().numpy() for k, v in o.items()}

    try:
        ctx.set_option(tg3.OPT_BANK_ORDER, order)
        a, b = run(form), run(1)
    finally:
        # the library's defaults
        ctx.set_option(tg3.OPT_BANK_GATHER, 0)
        ctx.set_option(tg3.OPT_BANK_ORDER, 1)
    assert np.max(np.abs(a["dvp"] - b["dvp"]) / np.abs(b["dvp"])) < 1e-5
    for l in range(n):
        assert np.argmax(a["dvp"][l]) == np.argmax(b["dvp"][l])
    qg = case["qg"]
    ix, tr = idx.cpu().numpy(), trans.cpu().numpy()
    for l in (0, 4, 7):
        c = int(ps.cls[l])
        vol = case["vols"][c].cpu().numpy().astype(np.complex128)
        ref = O.score_local(vol, case["pf"], ps.iCol, ps.iRow, case["box"],
                            ps.dat[l].cpu().numpy().astype(np.complex128),
                            ps.ctf[l].cpu().numpy().astype(np.float64),
                            ps.sigRcp[l].cpu().numpy().astype(np.float64), qg[ix[l]], tr[l],
                            np.full(nR, 1.0 / nR), np.full(nT, 1.0 / nT))
        assert np.max(np.abs(a["dvp"][l] - ref["dvp"]) / np.abs(ref["dvp"])) < 1e-4
        assert np.argmax(a["dvp"][l]) == np.argmax(ref["dvp"])
        for k in ("wR", "wT"):
            assert np.abs(a[k][l] / a[k][l].sum() - ref[k] / ref[k].sum()).max() < 2e-3


def test_reference_rendering_matches_the_torch_form():
    """tg3_ctx_render_references_d (projection over the image's rfft grid,
    cuFFT C2R, centring, normalisation, all in the library) against the
    same steps written with the context's projection and torch.fft: equal
    to float32 rounding, and the context's pixel set untouched."""
    rng = np.random.default_rng(12)
    box, px, pf, img = 128, 1.4, 2, 64
    bm = synth.blob_map(rng, 60, (1.5, 3.0), px, 40.0)
    ctx = tg3.Context(0)
    try:
        ctx.set_volume(0, synth.padded_volume(bm, box, pf, device=DEV, dtype=torch.float32), pf)
        q = synth.haar_quaternions(rng, 37)
        got = learned.render_references(ctx, 0, q, box, img)
        iCol, iRow = learned.image_grid(img)
        ctx.set_pixels(iCol, iRow, box)
        R = torch.as_tensor(synth.quat_to_mat(q).reshape(len(q), 9)).to(DEV)
        P = torch.empty((len(q), len(iCol)), dtype=torch.complex64, device=DEV)
        ctx.project(0, R, len(q), P)
        ctx.sync()
        ims = torch.fft.irfft2(P.view(len(q), img, img // 2 + 1), s=(img, img))
        ims = torch.fft.fftshift(ims, dim=(-2, -1))
        ims = ims - ims.mean(dim=(-2, -1), keepdim=True)
        want = ims / ims.std(dim=(-2, -1), keepdim=True)
        assert torch.isfinite(got).all()
        assert (got - want).abs().max().item() < 1e-4
    finally:
        ctx.close()


@pytest.mark.parametrize("shape", [0, 1, 2])
@pytest.mark.parametrize("nR", [32, 160])
def test_bank_pipeline_shapes(case, nR, shape):
    """The cp.async bank-row cross term's pipeline shapes (TG3_OPT_BANK_SHAPE:
    0 eight gather warps, 1 K blocks of 32 bf16 with twice the stages, 2 K
    blocks of 32 with two CTAs an SM) against the default (3: K blocks of 64,
    sixteen gather warps): the same MMAs in the same order and the norms
    summed over other lane partitions, so log-likelihoods within 1e-6
    relative and the same best hypothesis."""
    ps, ctx, n = case["ps"], case["ctx"], len(case["ps"].cls)
    nT = 9
    rng = np.random.default_rng(nR + 7)
    idx = torch.as_tensor(rng.integers(0, len(case["qg"]), (n, nR)).astype(np.int32), device=DEV)
    trans = torch.as_tensor(rng.uniform(-2, 2, (n, nT, 2)), **F64)

    def run(sh):
        ctx.set_option(tg3.OPT_BANK_SHAPE, sh)
        dvp = torch.empty((n, nR, nT), dtype=torch.float32, device=DEV)
        o = [torch.empty(n, **F64), torch.empty((n, nR), **F64), torch.empty((n, nT), **F64),
             torch.empty(n, **F64)]
        ctx.local_phase_bank(n, nR, nT, ps.dat, ps.ctf, ps.sigRcp, idx, trans,
                             torch.full((n, nR), 1.0 / nR, **F64),
                             torch.full((n, nT), 1.0 / nT, **F64), torch.ones(n, **F64),
                             case["cls"], *o, dvp, tg3.SCORE_BF16X3)
        ctx.sync()
        return dvp.cpu().numpy().astype(np.float64)

    try:
        a, b = run(shape), run(3)
    finally:
        ctx.set_option(tg3.OPT_BANK_SHAPE, 3)
    assert np.max(np.abs(a - b) / np.abs(b)) < 1e-6
    for l in range(n):
        assert np.argmax(a[l]) == np.argmax(b[l])
