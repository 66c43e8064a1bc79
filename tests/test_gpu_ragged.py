"""Uneven batches: a ragged plan over particles of three classes, each class
with its own cutoff (pixel set), each particle with its own rotation and
translation counts, against every particle scored and resampled alone
through the batched entry points (one particle per call).  The plan pads
particles inside waves with zero-prior copies of their own hypotheses, which
must leave every output unchanged: the comparison is exact."""
import numpy as np
import pytest
import torch

import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"
BOX, PF, PX = 32, 2, 1.5
CUTOFFS = (8, 10, 12)


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(303)
    maps = synth.class_maps(rng, len(CUTOFFS), 0.7, 12, (2.0, 4.0), PX, 8.0)
    ctx = tg3.Context(0)
    for c, bm in enumerate(maps):
        ctx.set_volume(c, synth.padded_volume(bm, BOX, PF, device=DEV, dtype=torch.float32), PF)
    rL = synth.config_rL(BOX, PX)
    nP = 30
    cls = np.arange(nP) % len(CUTOFFS)
    nR = rng.integers(5, 71, nP)
    nT = rng.integers(2, 26, nP)
    pix, parts = [], []
    for c, rU in enumerate(CUTOFFS):
        st = synth.make_stack(400 + c, [maps[c]], BOX, PX, PF, rU, rL, nP, 2.0, 0.1)
        ctx.set_pixels_slot(c, st.iCol, st.iRow, BOX)
        pix.append(st)
    ctx.set_pixels(pix[0].iCol, pix[0].iRow, BOX)
    host = {k: [] for k in tg3.RAGGED_INPUTS}
    for l in range(nP):
        st = pix[cls[l]]
        q = synth.vmf_quaternions(rng, st.quat_true[l], 150.0, int(nR[l]))
        t = st.trans_true[l] + rng.standard_normal((int(nT[l]), 2))
        host["dat"].append(st.dat[l].astype(np.complex64))
        host["ctf"].append(st.ctf[l].astype(np.float32))
        host["sig"].append(st.sigRcp[l].astype(np.float32))
        host["quat"].append(q)
        host["trans"].append(t)
        host["pwR"].append(rng.random(int(nR[l])) + 0.1)
        host["pwT"].append(rng.random(int(nT[l])) + 0.1)
        host["pwC"].append(np.ones(1))
        host["permR"].append(rng.permutation(int(nR[l])).astype(np.int32))
        host["u0R"].append(rng.random(1) / nR[l])
        host["peakR"].append(np.full(1, np.nan))
        host["permT"].append(rng.permutation(int(nT[l])).astype(np.int32))
        host["u0T"].append(rng.random(1) / nT[l])
        host["peakT"].append(np.zeros(1))
    packed = {k: np.ascontiguousarray(np.concatenate(v)) for k, v in host.items()}
    dev = {k: torch.as_tensor(v).to(DEV) for k, v in packed.items()}
    yield dict(ctx=ctx, cls=cls, nR=nR, nT=nT, dev=dev, K=[p.K for p in pix])
    ctx.close()


def _outputs(nP, nR, nT):
    R, T = int(nR.sum()), int(nT.sum())
    f64 = dict(dtype=torch.float64, device=DEV)
    i32 = dict(dtype=torch.int32, device=DEV)
    return dict(wC=torch.empty(nP, **f64), base=torch.empty(nP, **f64),
                wR=torch.empty(R, **f64), wT=torch.empty(T, **f64),
                srcR=torch.empty(R, **i32), wOutR=torch.empty(R, **f64),
                srcT=torch.empty(T, **i32), wOutT=torch.empty(T, **f64),
                topR=torch.empty(nP, **i32), topT=torch.empty(nP, **i32))


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3], ids=["fp32", "bf16x3"])
def test_ragged_plan_equals_particles_alone(setup, precision):
    ctx, cls, nR, nT, d = setup["ctx"], setup["cls"], setup["nR"], setup["nT"], setup["dev"]
    nP = len(cls)
    out = _outputs(nP, nR, nT)
    # a small budget forces several waves per class
    plan = tg3.RaggedPlan(ctx, cls, nR, nT, d, out, precision, budget=96 << 10, graph=True)
    waves, _ = plan.info()
    assert waves > len(CUTOFFS)
    plan.run()
    ctx.sync()
    got = {k: v.cpu().numpy() for k, v in out.items()}
    plan.close()
    # every particle alone
    ref = _outputs(nP, nR, nT)
    po = ro = to = 0
    for l in range(nP):
        K, r, t = setup["K"][cls[l]], int(nR[l]), int(nT[l])
        ctx.use_pixels(int(cls[l]))
        sl = lambda k, a, n: d[k][a:a + n]
        dat = d["dat"][po:po + K]
        cl = torch.tensor([cls[l]], dtype=torch.int32, device=DEV)
        ctx.local_phase(1, r, t, dat, sl("ctf", po, K), sl("sig", po, K),
                        d["quat"][ro:ro + r], d["trans"][to:to + t], sl("pwR", ro, r),
                        sl("pwT", to, t), sl("pwC", l, 1), cl, ref["wC"][l:l + 1],
                        ref["wR"][ro:ro + r], ref["wT"][to:to + t], ref["base"][l:l + 1], None,
                        precision)
        ctx.resample(1, r, ref["wR"][ro:ro + r], sl("pwR", ro, r), sl("permR", ro, r),
                     sl("u0R", l, 1), sl("peakR", l, 1), r, ref["srcR"][ro:ro + r],
                     ref["wOutR"][ro:ro + r], ref["topR"][l:l + 1])
        ctx.resample(1, t, ref["wT"][to:to + t], sl("pwT", to, t), sl("permT", to, t),
                     sl("u0T", l, 1), sl("peakT", l, 1), t, ref["srcT"][to:to + t],
                     ref["wOutT"][to:to + t], ref["topT"][l:l + 1])
        ctx.sync()
        po, ro, to = po + K, ro + r, to + t
    ctx.use_pixels(-1)
    exp = {k: v.cpu().numpy() for k, v in ref.items()}
    for k in tg3.RAGGED_OUTPUTS:
        assert np.array_equal(got[k], exp[k]), k


def test_autotuned_plan_matches_a_fixed_plan(setup):
    """A plan whose budget, cross-term K block and projection rotations per CTA
    the autotuner chose (tg3_ragged_plan_kblock and _project_group report
    them) gives the same outputs as a plan with a fixed budget: waves, K blocks
    and projection tiles change the launches, not the arithmetic."""
    ctx, cls, nR, nT, d = setup["ctx"], setup["cls"], setup["nR"], setup["nT"], setup["dev"]
    nP = len(cls)
    res = []
    for budget in (0, 96 << 10):
        out = _outputs(nP, nR, nT)
        plan = tg3.RaggedPlan(ctx, cls, nR, nT, d, out, tg3.SCORE_BF16X3, budget=budget,
                              graph=True)
        assert plan.kblock() in (32, 64)
        assert plan.project_group() in (4, 8, 16)
        plan.run()
        ctx.sync()
        res.append({k: v.cpu().numpy() for k, v in out.items()})
        plan.close()
    for k in res[0]:
        np.testing.assert_array_equal(res[0][k], res[1][k])
