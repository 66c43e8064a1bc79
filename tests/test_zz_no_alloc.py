"""The allocation-free local scoring entry point (tg3_local_phase_noalloc)
against the regular one (tg3_local_phase_d) on the same inputs.

The allocation-free form exists for callers that cannot let the library
allocate device memory -- an application whose own pool allocator owns the
GPU's memory, or one that scores from many host threads, where each
cudaMalloc / cudaFree would synchronise the device.  It keeps its scratch in
a fixed device array of the library; this test checks that two calls in a
row (the second reusing the scratch the first left behind) both match the
regular entry point, within the tolerances of the other parity tests.

Runs last in the suite (file name), so a failure here leaves every other
test already run; it also passes when run alone in a fresh process."""
import numpy as np
import pytest
import torch

import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _case(seed, box=32, pf=2, px=1.5, rU=12, nR=80, nT=15):
    rng = np.random.default_rng(seed)
    rL = synth.config_rL(box, px)
    bm = synth.blob_map(rng, 20, (2.0, 4.0), px, 9.0)
    vol = synth.padded_volume(bm, box, pf).numpy().astype(np.complex64)
    st = synth.make_stack(seed + 1, [bm], box, px, pf, rU, rL, 1, 2.0, 0.5)
    qs, ts = synth.local_hypotheses(rng, st.quat_true, st.trans_true, nR, nT, 200.0, 1.0)
    return dict(box=box, pf=pf, vol=vol, st=st, q=qs[0], t=ts[0],
                pwR=rng.random(nR) + 0.5, pwT=rng.random(nT) + 0.5, nR=nR, nT=nT)


def _edge_case(seed=404, box=32, nR=40, nT=9):
    """Padding 1 with every pixel within radius 15 of a box-32 image: the
    pixel (0, 15) at the identity rotation samples row y0 = 15 = vdim / 2 - 1,
    whose upper corner is the stored Nyquist row; both entry points must take it."""
    import dataclasses
    c = _case(seed, box=box, pf=1, rU=16, nR=nR, nT=nT)
    st = c["st"]
    keep = np.nonzero(st.iCol.astype(np.int64) ** 2 + st.iRow.astype(np.int64) ** 2 <= 225)[0]
    assert np.any((st.iCol[keep] == 0) & (st.iRow[keep] == 15))
    c["st"] = dataclasses.replace(st, iCol=st.iCol[keep], iRow=st.iRow[keep], iSig=st.iSig[keep],
                                  ctf=st.ctf[:, keep], dat=st.dat[:, keep],
                                  sigRcp=st.sigRcp[:, keep])
    c["q"] = c["q"].copy()
    c["q"][0] = (1.0, 0.0, 0.0, 0.0)
    return c


def _dev(x):
    return torch.as_tensor(np.ascontiguousarray(x)).to(DEV)


def _outs(nR, nT):
    return dict(wC=torch.empty(1, dtype=torch.float64, device=DEV),
                wR=torch.empty(nR, dtype=torch.float64, device=DEV),
                wT=torch.empty(nT, dtype=torch.float64, device=DEV),
                base=torch.empty(1, dtype=torch.float64, device=DEV),
                dvp=torch.empty((nR, nT), dtype=torch.float32, device=DEV))


def _regular(c):
    st = c["st"]
    ctx = tg3.Context(0)
    try:
        ctx.set_volume(0, _dev(c["vol"]), c["pf"])
        ctx.set_pixels(st.iCol, st.iRow, c["box"])
        o = _outs(c["nR"], c["nT"])
        ctx.local_phase(1, c["nR"], c["nT"], _dev(st.dat.astype(np.complex64)),
                        _dev(st.ctf.astype(np.float32)), _dev(st.sigRcp.astype(np.float32)),
                        _dev(c["q"][None]), _dev(c["t"][None]), _dev(c["pwR"][None]),
                        _dev(c["pwT"][None]), _dev(np.ones(1)), None, o["wC"], o["wR"],
                        o["wT"], o["base"], o["dvp"])
        ctx.sync()
        return {k: v.cpu().numpy() for k, v in o.items()}
    finally:
        ctx.close()


def _noalloc(c):
    st = c["st"]
    ins = dict(vol=_dev(c["vol"]), iCol=_dev(st.iCol), iRow=_dev(st.iRow),
               dat=_dev(st.dat[0].astype(np.complex64)), ctf=_dev(st.ctf[0].astype(np.float32)),
               sig=_dev(st.sigRcp[0].astype(np.float32)), q=_dev(c["q"]), t=_dev(c["t"]),
               pwR=_dev(c["pwR"]), pwT=_dev(c["pwT"]))
    o = _outs(c["nR"], c["nT"])
    torch.cuda.synchronize()
    p = tg3.ptr
    tg3.check(tg3.lib().tg3_local_phase_noalloc(
        p(ins["vol"]), c["vol"].shape[0], c["pf"], p(ins["iCol"]), p(ins["iRow"]), len(st.iCol),
        c["box"],
        p(ins["dat"]), p(ins["ctf"]), p(ins["sig"]), p(ins["q"]), c["nR"], p(ins["t"]), c["nT"],
        p(ins["pwR"]), p(ins["pwT"]), None, p(o["wC"]), p(o["wR"]), p(o["wT"]), p(o["base"]),
        p(o["dvp"]), None))
    return {k: v.cpu().numpy() for k, v in o.items()}


def _agree(a, b):
    # the parity tolerances of the FP32 path
    assert np.max(np.abs(a["dvp"] - b["dvp"]) / np.abs(b["dvp"])) < 1e-4
    assert abs(a["base"][0] - b["base"][0]) / abs(b["base"][0]) < 1e-4
    assert np.argmax(a["dvp"]) == np.argmax(b["dvp"])
    for k in ("wR", "wT"):
        assert np.abs(a[k] / a[k].sum() - b[k] / b[k].sum()).max() < 2e-3
    assert abs(a["wC"][0] - b["wC"][0]) / b["wC"][0] < 5e-2


def test_noalloc_matches_regular_entry_twice():
    first = _case(101)
    second = _case(202, nR=120, nT=9)      # a different shape reuses the scratch
    _agree(_noalloc(first), _regular(first))
    _agree(_noalloc(second), _regular(second))


def test_noalloc_samples_the_nyquist_row():
    c = _edge_case()
    _agree(_noalloc(c), _regular(c))


def test_noalloc_rejects_oversized_sets():
    c = _case(303, nR=8, nT=4)
    cap = tg3.lib().tg3_noalloc_scratch_bytes()
    st = c["st"]
    kp = ((2 * st.K + 63) // 64) * 64
    nR = cap // (4 * kp) + 1                 # projection bank alone exceeds the scratch
    q = np.tile(c["q"][:1], (nR, 1))
    dq, dt = _dev(q), _dev(c["t"])
    dummy = torch.zeros(8, dtype=torch.float64, device=DEV)
    p = tg3.ptr
    rc = tg3.lib().tg3_local_phase_noalloc(
        p(_dev(c["vol"])), c["vol"].shape[0], c["pf"], p(_dev(st.iCol)), p(_dev(st.iRow)), st.K,
        c["box"], p(_dev(st.dat[0].astype(np.complex64))), p(_dev(st.ctf[0].astype(np.float32))),
        p(_dev(st.sigRcp[0].astype(np.float32))), p(dq), nR, p(dt), c["nT"], p(dummy), p(dummy),
        None, p(dummy), p(dummy), p(dummy), p(dummy), None, None)
    assert rc == tg3.ERR_ARG
    assert b"fixed scratch" in tg3.lib().tg3_last_error()
