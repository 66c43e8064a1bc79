"""Split-precision scoring at production size against the FP64 oracle: box 256,
three classes whose maps share 70 % of their 200 blobs, cutoff 120 (K = 22,422),
local hypotheses (vMF kappa 200 rotations, Gaussian translations).

For two particles of every class, the per-hypothesis log-likelihoods of the
plain FP32 path and of the split-bf16 tcgen05 path are compared with the
oracle's on the same inputs (the FP32 class volumes, read in double by the
oracle).  Bars: 1e-4 relative for every log-likelihood and the same best
hypothesis as the oracle for both paths."""
import numpy as np
import pytest
import torch

import tg3
from tg3 import synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DEV = "cuda:0"
BOX, PF, PX = 256, 2, 1.1
N_CLASSES, SHARED = 3, 0.7
NR, NT = 44, 100          # 5 full rotation groups of 8 and a partial one
PER_CLASS = 2


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(2002)
    maps = synth.class_maps(rng, N_CLASSES, SHARED, 200, (1.5, 3.0), PX, 80.0)
    vols = [synth.padded_volume(bm, BOX, PF, device=DEV, dtype=torch.float32) for bm in maps]
    rL = synth.config_rL(BOX, PX)
    n = N_CLASSES * PER_CLASS
    st = synth.make_stack(2003, maps, BOX, PX, PF, 120, rL, n, 8.0, 0.03, device=DEV)
    assert st.K == 22422
    qc, tc = synth.perturb_poses(rng, st.quat_true, st.trans_true, 3.0, 1.0)
    qs, ts = synth.local_hypotheses(rng, qc, tc, NR, NT, 200.0, 2.0)
    ctx = tg3.Context(0)
    for c, v in enumerate(vols):
        ctx.set_volume(c, v, PF)
    ctx.set_pixels(st.iCol, st.iRow, BOX)
    host_vols = [v.cpu().numpy().astype(np.complex128) for v in vols]
    del vols
    yield dict(ctx=ctx, st=st, qs=qs, ts=ts, vols=host_vols, n=n)
    ctx.close()


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3], ids=["fp32", "bf16x3"])
def test_three_class_cutoff120_against_oracle(setup, precision):
    st, n = setup["st"], setup["n"]
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    dat = torch.as_tensor(st.dat.astype(np.complex64)).to(DEV)
    ctf = torch.as_tensor(f32(st.ctf)).to(DEV)
    sig = torch.as_tensor(f32(st.sigRcp)).to(DEV)
    quat = torch.as_tensor(setup["qs"]).to(DEV)
    trans = torch.as_tensor(setup["ts"]).to(DEV)
    pwR = torch.full((n, NR), 1.0 / NR, dtype=torch.float64, device=DEV)
    pwT = torch.full((n, NT), 1.0 / NT, dtype=torch.float64, device=DEV)
    pwC = torch.ones(n, dtype=torch.float64, device=DEV)
    cls = torch.as_tensor(st.cls_true.astype(np.int32)).to(DEV)
    wC = torch.empty(n, dtype=torch.float64, device=DEV)
    wR = torch.empty((n, NR), dtype=torch.float64, device=DEV)
    wT = torch.empty((n, NT), dtype=torch.float64, device=DEV)
    base = torch.empty(n, dtype=torch.float64, device=DEV)
    dvp = torch.empty((n, NR, NT), dtype=torch.float32, device=DEV)
    ctx = setup["ctx"]
    ctx.local_phase(n, NR, NT, dat, ctf, sig, quat, trans, pwR, pwT, pwC, cls, wC, wR, wT, base,
                    dvp, precision)
    ctx.sync()
    g = dvp.cpu().numpy()
    worst = 0.0
    for l in range(n):
        r = O.score_local(setup["vols"][st.cls_true[l]], PF, st.iCol, st.iRow, BOX,
                          st.dat[l].astype(np.complex64), f32(st.ctf[l]), f32(st.sigRcp[l]),
                          setup["qs"][l], setup["ts"][l], np.full(NR, 1.0 / NR),
                          np.full(NT, 1.0 / NT), 1.0)
        rel = np.abs(g[l] - r["dvp"]) / np.abs(r["dvp"])
        worst = max(worst, float(rel.max()))
        assert rel.max() < 1e-4, (l, rel.max())
        assert np.argmax(g[l]) == np.argmax(r["dvp"])
    print(f"\nconfig-2 {'fp32' if precision == tg3.SCORE_FP32 else 'bf16x3'}: "
          f"max relative log-likelihood error vs the FP64 oracle {worst:.3e}")
