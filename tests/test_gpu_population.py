"""Population parity: the best hypothesis of every particle against the FP64
oracle, at the sizes of the E-step's configurations.

The acceptance bar is the same argmax pose (rotation x translation) as the
FP64 oracle for >= 99.9 % of particles, on a population rather than a
handful:
- configuration 0 in full: box 64, 2,000 particles, the global search over
  6,912 rotations x 49 translations (K = 375), FP32 and split-bf16;
- configuration 1 on a subset: box 256, K = 9,930, local phases of 1,000
  rotations x 100 translations, 128 particles, FP32 and split-bf16.
Beside the argmax the tests bound the error of the log-likelihood
differences L - max L over the hypotheses within 30 of the best (those with
non-negligible weight): a whole-likelihood relative bar of 1e-4 alone would
allow absolute errors of several units there.

The oracle's projections come from the C restatement (or_project, pinned to
the compiled reference); the likelihoods use the expansion
L(r, t) = x0 + sum_p sigRcp c^2 |P_r|^2 - 2 Re sum_p sigRcp c conj(X) S_t P_r
in float64, which is checked here against the C oracle's own global scan
(or_score_global) on a few particles first.  The oracle sees the
float32-rounded inputs the GPU sees."""
import multiprocessing as mp
import os
import tempfile
from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import oracle as O
import tg3
from tg3 import synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
F64 = dict(dtype=torch.float64, device=DEV)
ROOT = Path(__file__).resolve().parents[1]


def f32(x):
    x = np.asarray(x)
    if np.iscomplexobj(x):
        return x.astype(np.complex64).astype(np.complex128)
    return x.astype(np.float32).astype(np.float64)


def likelihoods(P, S, X, c, s):
    """FP64 log-likelihoods [nR][nT] of one image X (K complex) with CTF c and
    sigRcp s against projections P [nR][K] and phase shifts S [nT][K]."""
    x0 = float(np.sum(s * np.abs(X) ** 2))
    nrm = (np.abs(P) ** 2) @ (s * c * c)
    A = (s * c * np.conj(X))[None, :] * S
    return x0 + nrm[:, None] - 2.0 * np.real(A @ P.T).T


def likelihoods_batch(P, S, X, c, s):
    """likelihoods for a batch of images X [n][K] (c, s [n][K]): [n][nR][nT],
    the cross term as one real GEMM over the stacked real and imaginary parts."""
    n, nT = X.shape[0], S.shape[0]
    x0 = np.sum(s * np.abs(X) ** 2, axis=1)                          # [n]
    nrm = (np.abs(P) ** 2) @ (s * c * c).T                            # [nR][n]
    A = ((s * c * np.conj(X))[:, None, :] * S[None, :, :]).reshape(n * nT, -1)
    cross = np.concatenate([A.real, -A.imag], 1) @ np.concatenate([P.real, P.imag], 1).T
    cross = cross.reshape(n, nT, -1).transpose(0, 2, 1)               # [n][nR][nT]
    return x0[:, None, None] + nrm.T[:, :, None] - 2.0 * cross


def compare(dvp_gpu, L64):
    """(same argmax, max |dL error| within 30 of the best, oracle shortfall
    of the GPU's pick in units of L)."""
    g = dvp_gpu.reshape(-1).astype(np.float64)
    o = L64.reshape(-1)
    ig, io = int(np.argmax(g)), int(np.argmax(o))
    dg, do = g - g[ig], o - o[io]
    near = do > -30.0
    return ig == io, float(np.abs(dg - do)[near].max()), float(o[io] - o[ig])


@pytest.fixture(scope="module")
def config0():
    rng = np.random.default_rng(1000)
    box, px, pf, rU = 64, 1.5, 2, 16
    bm = synth.blob_map(rng, 40, (2.0, 4.0), px, 20.0)
    rL = synth.config_rL(box, px)
    st = synth.make_stack(2000, [bm], box, px, pf, rU, rL, 2000, 3.0, 0.05)
    vol32 = synth.padded_volume(bm, box, pf, device=DEV, dtype=torch.float32)
    q = synth.global_rotations(4, 36)
    trans = synth.global_translations(3, 1.0)
    return dict(box=box, pf=pf, st=st, vol32=vol32, vol=f32(vol32.cpu().numpy()), q=q, trans=trans)


@pytest.mark.parametrize("precision", [tg3.SCORE_FP32, tg3.SCORE_BF16X3])
def test_config0_global_search_population(config0, precision):
    c0 = config0
    st, q, trans = c0["st"], c0["q"], c0["trans"]
    n, nR, nT, K = len(st.dat), len(q), len(trans), st.K
    mats = synth.quat_to_mat(q).reshape(-1, 9)
    dat, ctf, sig = (st.dat.astype(np.complex64), st.ctf.astype(np.float32),
                     st.sigRcp.astype(np.float32))
    ctx = tg3.Context(0)
    try:
        ctx.set_volume(0, c0["vol32"], c0["pf"])
        ctx.set_pixels(st.iCol, st.iRow, c0["box"])
        o = dict(wC=torch.empty(n, **F64), wR=torch.empty((n, nR), **F64),
                 wT=torch.empty((n, nT), **F64), base=torch.empty(n, **F64),
                 dvp=torch.empty((n, nR, nT), dtype=torch.float32, device=DEV))
        d = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(DEV)
        ctx.global_scan(0, n, nR, nT, d(dat), d(ctf), d(sig), d(mats), d(trans),
                        torch.full((nR,), 1.0 / nR, **F64), torch.full((nT,), 1.0 / nT, **F64),
                        o["wC"], o["wR"], o["wT"], o["base"], o["dvp"], precision)
        ctx.sync()
        dvp = o["dvp"]
        # the oracle: projections, phase shifts; the expansion checked against
        # the C global scan on two particles
        P = O.project(c0["vol"], mats, st.iCol, st.iRow, c0["pf"])
        S = O.translate(f32(trans), c0["box"], st.iCol, st.iRow)
        X, C, Sg = f32(dat), f32(ctf), f32(sig)
        ref = O.score_global(P, S, X[:2], C[:2], Sg[:2], np.full(nR, 1.0 / nR),
                             np.full(nT, 1.0 / nT))["dvp"]
        Lb = likelihoods_batch(P, S, X[:2], C[:2], Sg[:2])
        for l in range(2):
            assert np.max(np.abs(Lb[l] - ref[l]) / np.abs(ref[l])) < 1e-12
            assert np.max(np.abs(likelihoods(P, S, X[l], C[l], Sg[l]) - ref[l])
                          / np.abs(ref[l])) < 1e-12
        same, err_near, shortfall = 0, 0.0, []
        for s0 in range(0, n, 200):
            g = dvp[s0:s0 + 200].cpu().numpy()
            Lc = likelihoods_batch(P, S, X[s0:s0 + 200], C[s0:s0 + 200], Sg[s0:s0 + 200])
            for j in range(len(g)):
                eq, e, sh = compare(g[j], Lc[j])
                same += eq
                err_near = max(err_near, e)
                if not eq:
                    shortfall.append(sh)
    finally:
        ctx.close()
    frac = same / n
    print(f"config 0, precision {precision}: same argmax {frac:.5f} ({n - same} of {n} differ; "
          f"oracle shortfall of the GPU's pick {shortfall}); max |dL error| within 30 of the "
          f"best {err_near:.4g}")
    assert frac >= 0.999, (frac, shortfall)
    # the differences that decide the weights: a fraction of a unit of L
    assert err_near < (0.05 if precision == tg3.SCORE_FP32 else 0.25), err_near


def _config1_worker(job):
    """One particle of configuration 1: the oracle's projections of its
    rotations and its FP64 likelihoods, compared with the GPU's (both
    precisions)."""
    import sys as _s
    for p in job["paths"]:
        if p not in _s.path:
            _s.path.insert(0, p)
    from oracle import oracle as O
    vol = np.load(job["vol"], mmap_mode="r")
    P = O.project(np.asarray(vol), job["mats"], job["iCol"], job["iRow"], job["pf"])
    S = O.translate(job["trans"], job["box"], job["iCol"], job["iRow"])
    L = likelihoods(P, S, job["X"], job["c"], job["s"])
    return [compare(g, L) for g in job["dvp"]] + [float(np.max(np.abs(
        job["dvp"][0].astype(np.float64) - L) / np.abs(L)))]


def test_config1_local_phase_population():
    rng = np.random.default_rng(1001)
    box, px, pf, rU = 256, 1.1, 2, 80
    nP, nR, nT = 128, 1000, 100
    bm = synth.blob_map(rng, 200, (1.5, 3.0), px, 80.0)
    rL = synth.config_rL(box, px)
    st = synth.make_stack(2001, [bm], box, px, pf, rU, rL, nP, 8.0, 0.03, device=DEV)
    qc, tc = synth.perturb_poses(rng, st.quat_true, st.trans_true, 3.0, 1.0)
    qs, ts = synth.local_hypotheses(rng, qc, tc, nR, nT, 200.0, 2.0)
    qs, ts = f32(qs), f32(ts)
    vol32 = synth.padded_volume(bm, box, pf, device=DEV, dtype=torch.float32)
    dat, ctf, sig = (st.dat.astype(np.complex64), st.ctf.astype(np.float32),
                     st.sigRcp.astype(np.float32))
    d = lambda x: torch.as_tensor(np.ascontiguousarray(x)).to(DEV)
    ctx = tg3.Context(0)
    dvps = []
    try:
        ctx.set_volume(0, vol32, pf)
        ctx.set_pixels(st.iCol, st.iRow, box)
        for precision in (tg3.SCORE_FP32, tg3.SCORE_BF16X3):
            o = dict(wC=torch.empty(nP, **F64), wR=torch.empty((nP, nR), **F64),
                     wT=torch.empty((nP, nT), **F64), base=torch.empty(nP, **F64),
                     dvp=torch.empty((nP, nR, nT), dtype=torch.float32, device=DEV))
            ctx.local_phase(nP, nR, nT, d(dat), d(ctf), d(sig), d(qs), d(ts),
                            torch.full((nP, nR), 1.0 / nR, **F64),
                            torch.full((nP, nT), 1.0 / nT, **F64), torch.ones(nP, **F64), None,
                            o["wC"], o["wR"], o["wT"], o["base"], o["dvp"], precision)
            ctx.sync()
            dvps.append(o["dvp"].cpu().numpy())
    finally:
        ctx.close()
    tmp = tempfile.mkdtemp()
    vpath = os.path.join(tmp, "vol.npy")
    np.save(vpath, f32(vol32.cpu().numpy()))
    del vol32
    paths = [str(ROOT), str(ROOT / "thunder-refactor-expectation_gb300")]
    jobs = [dict(vol=vpath, mats=O.rotmat(qs[l]).reshape(-1, 9), trans=ts[l], iCol=st.iCol,
                 iRow=st.iRow, pf=pf, box=box, X=f32(dat[l]), c=f32(ctf[l]), s=f32(sig[l]),
                 dvp=[dvps[0][l], dvps[1][l]], paths=paths) for l in range(nP)]
    # one BLAS thread per worker process (they read the setting when they start)
    saved = {k: os.environ.get(k) for k in ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS")}
    os.environ.update(OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    try:
        with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
            res = pool.map(_config1_worker, jobs)
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        os.unlink(vpath)
        os.rmdir(tmp)
    for k, name in enumerate(("fp32", "bf16x3")):
        same = sum(r[k][0] for r in res)
        err = max(r[k][1] for r in res)
        print(f"config 1 subset, {name}: same argmax {same} of {nP}; max |dL error| within 30 "
              f"of the best {err:.4g}")
        assert same / nP >= 0.999, (name, same)
        assert err < (0.05 if k == 0 else 0.25), (name, err)
    # whole log-likelihoods of the FP32 path within 1e-4 relative
    assert max(r[-1] for r in res) < 1e-4
