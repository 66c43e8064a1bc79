"""Learned proposal: training the pose network and drawing hypotheses from it.

The network (tg3.Cnn, all kernels the library's own) runs in one of two
modes on a particle's 64 x 64 image:
- regression: outputs a mixture of 8 rotations (6-D representation,
  concentration, weight) and a Gaussian shift; proposals are drawn from it;
- matching: outputs an embedding (compared by cosine with the embeddings of
  clean reference projections of the particle's map) and the same Gaussian
  shift; proposals are the best-matching reference rotations.
Either way the proposals seed the particle filter in place of the uniform
global initialisation: every proposed hypothesis is rescored by the exact
likelihood (tg3_local_phase_d), and the plain global search remains the
fallback.
"""
from __future__ import annotations

import math

import numpy as np

from . import synth

N_COMP = 8


def _softplus(x):
    return np.where(x > 20, x, np.log1p(np.exp(np.minimum(x, 20))))


def decode(out: np.ndarray):
    """Network outputs [n][68] -> rotations [n][8][3][3], concentrations
    [n][8], weights [n][8], shift mean [n][2], shift deviation [n][2]."""
    n = out.shape[0]
    comp = out[:, :64].astype(np.float64).reshape(n, N_COMP, 8)
    a1, a2 = comp[..., 0:3], comp[..., 3:6]
    b1 = a1 / (np.linalg.norm(a1, axis=-1, keepdims=True) + 1e-12)
    u2 = a2 - (b1 * a2).sum(-1, keepdims=True) * b1
    b2 = u2 / (np.linalg.norm(u2, axis=-1, keepdims=True) + 1e-12)
    R = np.stack([b1, b2, np.cross(b1, b2)], -1)      # columns b1 b2 b3
    kap = _softplus(comp[..., 6]) + 1e-3
    lg = comp[..., 7]
    w = np.exp(lg - lg.max(1, keepdims=True))
    w /= w.sum(1, keepdims=True)
    mu = out[:, 64:66].astype(np.float64)
    sd = np.exp(0.5 * out[:, 66:68].astype(np.float64))
    return R, kap, w, mu, sd


def mat_to_quat(R: np.ndarray) -> np.ndarray:
    """Rotation matrices [..., 3, 3] -> unit quaternions (w, x, y, z), w >= 0."""
    m = R.reshape(-1, 3, 3)
    tr = m[:, 0, 0] + m[:, 1, 1] + m[:, 2, 2]
    q = np.empty((len(m), 4))
    q[:, 0] = np.sqrt(np.maximum(0.0, 1 + tr)) / 2
    q[:, 1] = np.sqrt(np.maximum(0.0, 1 + m[:, 0, 0] - m[:, 1, 1] - m[:, 2, 2])) / 2
    q[:, 2] = np.sqrt(np.maximum(0.0, 1 - m[:, 0, 0] + m[:, 1, 1] - m[:, 2, 2])) / 2
    q[:, 3] = np.sqrt(np.maximum(0.0, 1 - m[:, 0, 0] - m[:, 1, 1] + m[:, 2, 2])) / 2
    q[:, 1] = np.copysign(q[:, 1], m[:, 2, 1] - m[:, 1, 2])
    q[:, 2] = np.copysign(q[:, 2], m[:, 0, 2] - m[:, 2, 0])
    q[:, 3] = np.copysign(q[:, 3], m[:, 1, 0] - m[:, 0, 1])
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.reshape(R.shape[:-2] + (4,))


def _axis_angle(v: np.ndarray) -> np.ndarray:
    """Rotation vectors [..., 3] -> matrices [..., 3, 3] (Rodrigues)."""
    th = np.linalg.norm(v, axis=-1, keepdims=True)
    k = v / np.maximum(th, 1e-12)
    K = np.zeros(v.shape[:-1] + (3, 3))
    K[..., 0, 1], K[..., 0, 2], K[..., 1, 2] = -k[..., 2], k[..., 1], -k[..., 0]
    K[..., 1, 0], K[..., 2, 0], K[..., 2, 1] = k[..., 2], -k[..., 1], k[..., 0]
    th = th[..., None]
    return np.eye(3) + np.sin(th) * K + (1 - np.cos(th)) * (K @ K)


def propose(out: np.ndarray, n_rot: int, n_trans: int, rng: np.random.Generator):
    """Hypotheses drawn from the network's outputs: quaternions [n][n_rot][4]
    (component counts from the mixture weights, each sample the component's
    rotation turned by a rotation vector ~ N(0, I / kappa)) and translations
    [n][n_trans][2] ~ N(mu, sd^2).  The component centres are always kept."""
    R, kap, w, mu, sd = decode(out)
    n = len(out)
    # component of every extra sample by inverse CDF of the mixture weights
    cdf = np.cumsum(w, 1)
    u = rng.random((n, n_rot - N_COMP)) * cdf[:, -1:]
    c = np.minimum((u[:, :, None] > cdf[:, None, :]).sum(-1), N_COMP - 1)
    comp = np.concatenate([np.broadcast_to(np.arange(N_COMP), (n, N_COMP)), c], 1)
    Rc = R[np.arange(n)[:, None], comp]                      # [n][n_rot][3][3]
    v = rng.standard_normal((n, n_rot, 3)) / np.sqrt(kap[np.arange(n)[:, None], comp])[..., None]
    v[:, :N_COMP] = 0.0
    Rs = Rc @ _axis_angle(v)
    quat = mat_to_quat(Rs)
    trans = mu[:, None, :] + sd[:, None, :] * rng.standard_normal((n, n_trans, 2))
    trans[:, 0] = mu
    return np.ascontiguousarray(quat), np.ascontiguousarray(trans)


def angle_deg(q1: np.ndarray, q2: np.ndarray) -> np.ndarray:
    d = np.abs((q1 * q2).sum(-1)).clip(0.0, 1.0)
    return np.degrees(2.0 * np.arccos(d))


def train(net, images, Rstar, tstar, epochs: int, batch: int, lr: float, seed: int = 0,
          log=None):
    """Minibatch Adam on (image, true pose) pairs: images [n][64][64],
    Rstar [n][9], tstar [n][2] (device tensors).  Cosine-decayed learning
    rate; returns the mean loss of every epoch."""
    import torch
    n = images.shape[0]
    rng = np.random.default_rng(seed)
    steps = epochs * (n // batch)
    k = 0
    losses = []
    for e in range(epochs):
        order = torch.as_tensor(rng.permutation(n), device=images.device)
        tot = 0.0
        for s in range(n // batch):
            idx = order[s * batch:(s + 1) * batch]
            net.zero_grads()
            tot += net.loss(images[idx].contiguous(), Rstar[idx].contiguous(),
                            tstar[idx].contiguous(), grads=True)
            net.adam(lr * 0.5 * (1 + math.cos(math.pi * k / max(steps, 1))))
            k += 1
        losses.append(tot / max(n // batch, 1))
        if log:
            log(f"epoch {e}: loss {losses[-1]:.4f}")
    return losses


# --------------------------------------------------------------------------
# Matching mode: the same network embeds particle images and clean reference
# projections of the particle's map (outputs 0..63, compared by cosine), so
# its proposals follow the map it is given, not the maps it was trained on.
# --------------------------------------------------------------------------
def image_grid(img: int = 64):
    """(iCol, iRow) of the img x img image's rfft grid, rows in FFT order
    (the order of the particle images' transforms)."""
    h = img // 2
    jj = np.concatenate([np.arange(0, h), np.arange(-h, 0)])
    ii = np.arange(0, h + 1)
    J, I = np.meshgrid(jj, ii, indexing="ij")
    return I.ravel().astype(np.int32), J.ravel().astype(np.int32)


def render_references(ctx, cls: int, quats: np.ndarray, box: int, img: int = 64,
                      chunk: int = 4096):
    """Clean projections of the context's class-`cls` volume at `quats` over
    the img x img rfft grid at the box's frequencies, as the network sees
    particles: to real space, centred, zero mean and unit deviation
    (tg3_ctx_render_references_d, all on the device: projection, cuFFT
    C2R, centring and normalisation).  Returns a device float32 tensor
    [n][img][img]; the context's pixel set is left alone."""
    import torch
    del box  # the grid is in the volume's own frequencies
    dev = f"cuda:{torch.cuda.current_device()}"
    n = len(quats)
    out = torch.empty((n, img, img), dtype=torch.float32, device=dev)
    R = torch.as_tensor(synth.quat_to_mat(quats).reshape(n, 9)).to(dev).contiguous()
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        ctx.render_references(cls, R[s:s + m], m, img, out[s:s + m])
    ctx.sync()
    return out


def reference_embeddings(net, refs, chunk: int = 4096):
    """Normalised embeddings [n][64] of reference images [n][64][64] (the
    inference forward: bf16 activations on the tensor cores)."""
    import torch
    n = refs.shape[0]
    z = torch.empty((n, 64), dtype=torch.float32, device=refs.device)
    out = torch.empty((min(chunk, n), net.N_OUT), dtype=torch.float32, device=refs.device)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        net.infer(refs[s:s + m].contiguous(), out[:m])
        net.embed(out[:m], z[s:s + m])
    torch.cuda.synchronize()
    return z


class TrainingStalled(RuntimeError):
    """The matching loss did not leave its starting plateau in the first
    epoch (stall_check): the embeddings stayed uninformative."""


def train_match(net, images, refs, tstar, cls, epochs: int, batch: int, lr: float,
                tau: float = 0.1, seed: int = 0, log=None, warmup: float = 0.02,
                stall_check: bool = False):
    """Minibatch Adam on the matching loss: particle images [n][64][64] and
    the clean references at their true rotations [n][64][64], shifts tstar
    [n][2] (device tensors); every batch holds particles of one map
    (cls [n]), so its negatives are other poses of that map.  Learning rate
    ramped up linearly over the first `warmup` fraction of the steps, then
    cosine-decayed; returns the mean loss of every epoch.

    The gradient sums use atomics, so runs differ in the last bits, and a run
    can stay on the loss's starting plateau.  With stall_check, the first
    epoch ends in TrainingStalled when the mean loss of its last tenth of
    batches is above 0.95 of that of its first twentieth (the caller starts
    again from another initialisation)."""
    import torch
    rng = np.random.default_rng(seed)
    cls = np.asarray(cls)
    groups = [np.nonzero(cls == c)[0] for c in np.unique(cls)]
    per_epoch = sum(len(g) // batch for g in groups)
    steps = epochs * per_epoch
    dev = images.device
    outP = torch.empty((batch, net.N_OUT), dtype=torch.float32, device=dev)
    outR = torch.empty_like(outP)
    dP = torch.empty_like(outP)
    dR = torch.empty_like(outP)
    k = 0
    losses = []
    warm = max(1, int(warmup * steps))
    for e in range(epochs):
        batches = []
        for g in groups:
            p = rng.permutation(g)
            batches += [p[b * batch:(b + 1) * batch] for b in range(len(g) // batch)]
        order = rng.permutation(len(batches))
        tot = 0.0
        hist = []
        for bi in order:
            idx = torch.as_tensor(batches[bi], device=dev)
            ip, ir = images[idx].contiguous(), refs[idx].contiguous()
            net.forward(ip, outP)
            net.forward(ir, outR)
            net.zero_grads()
            v = net.contrastive(outP, outR, tstar[idx].contiguous(), tau, dP, dR)
            tot += v
            hist.append(v)
            net.backward(ip, dP)
            net.backward(ir, dR)
            net.adam(lr * min(1.0, (k + 1) / warm)
                     * 0.5 * (1 + math.cos(math.pi * k / max(steps, 1))))
            k += 1
        losses.append(tot / max(per_epoch, 1))
        if log:
            log(f"epoch {e}: loss {losses[-1]:.4f}")
        if stall_check and e == 0 and len(hist) >= 40:
            first = float(np.mean(hist[:max(1, len(hist) // 20)]))
            last = float(np.mean(hist[-max(1, len(hist) // 10):]))
            if last > 0.95 * first:
                raise TrainingStalled(f"first-epoch loss {first:.3f} -> {last:.3f}")
    return losses


# --------------------------------------------------------------------------
# The plain method's converged poses (the training labels, and the poses the
# proposals' errors are measured against): the global search, then local
# particle-filter phases that narrow around the current best pose.
# --------------------------------------------------------------------------
# (concentration of the rotations' vMF, deviation of the translations in
# pixels) of the local phases after the global search: the particle
# filter's narrowing as the poses converge
CONVERGE_SCHEDULE = ((200.0, 2.0), (1000.0, 0.7), (5000.0, 0.3))


def global_best(ctx, ps, quats_g, mats_g, trans_g, precision, batch: int = 2048):
    """Best rotation (quaternion) and translation of every particle of ps
    (a synth.ParticleSetDev; the context holds every class's volume and the
    likelihood's pixel set) by the global search over quats_g x trans_g with
    uniform priors: argmax of the rotation and translation marginals.
    Returns float64 device tensors [n][4], [n][2] and the best
    log-likelihoods [n]."""
    import torch
    dev = ps.dat.device
    n = len(ps.cls)
    nRg, nTg = len(quats_g), int(trans_g.shape[0])
    f64 = dict(dtype=torch.float64, device=dev)
    qg = torch.as_tensor(quats_g, **f64)
    pR = torch.full((nRg,), 1.0 / nRg, **f64)
    pT = torch.full((nTg,), 1.0 / nTg, **f64)
    q_best = torch.empty((n, 4), **f64)
    t_best = torch.empty((n, 2), **f64)
    base = torch.empty(n, **f64)
    for c in np.unique(ps.cls):
        sel = np.nonzero(ps.cls == c)[0]
        for s in range(0, len(sel), batch):
            idx = torch.as_tensor(sel[s:s + batch], device=dev)
            m = len(idx)
            wC = torch.empty(m, **f64)
            wR = torch.empty((m, nRg), **f64)
            wT = torch.empty((m, nTg), **f64)
            b = torch.empty(m, **f64)
            ctx.global_scan(int(c), m, nRg, nTg, ps.dat[idx].contiguous(),
                            ps.ctf[idx].contiguous(), ps.sigRcp[idx].contiguous(), mats_g,
                            trans_g, pR, pT, wC, wR, wT, b, None, precision)
            ctx.sync()
            q_best[idx] = qg[wR.argmax(1)]
            t_best[idx] = trans_g[wT.argmax(1)]
            base[idx] = b
    return q_best, t_best, base


def local_refine(ctx, ps, q_c, t_c, kappa, trans_sd, precision, gen, nR: int = 1000,
                 nT: int = 100, batch: int = 256, sel=None):
    """One local phase about the poses q_c [n][4], t_c [n][2] (device float64):
    nR vMF rotations (concentration kappa) x nT Gaussian translations
    (deviation trans_sd) per particle, scored with uniform priors; the best
    rotation and translation (argmax of the marginals) and the best
    log-likelihood.  `sel` (optional index array) restricts it to those
    particles of ps (q_c, t_c then have one row per selected particle)."""
    import torch
    dev = ps.dat.device
    rows = np.arange(len(ps.cls)) if sel is None else np.asarray(sel)
    n = len(rows)
    f64 = dict(dtype=torch.float64, device=dev)
    q_new = torch.empty((n, 4), **f64)
    t_new = torch.empty((n, 2), **f64)
    base = torch.empty(n, **f64)
    cls_all = torch.as_tensor(ps.cls.astype(np.int32), device=dev)
    for s in range(0, n, batch):
        e = min(n, s + batch)
        m = e - s
        idx = torch.as_tensor(rows[s:e], device=dev)
        qs, ts = synth.local_hypotheses_dev(gen, q_c[s:e], t_c[s:e], nR, nT, kappa, trans_sd)
        pwR = torch.full((m, nR), 1.0 / nR, **f64)
        pwT = torch.full((m, nT), 1.0 / nT, **f64)
        pwC = torch.ones(m, **f64)
        wC = torch.empty(m, **f64)
        wR = torch.empty((m, nR), **f64)
        wT = torch.empty((m, nT), **f64)
        b = torch.empty(m, **f64)
        ctx.local_phase(m, nR, nT, ps.dat[idx].contiguous(), ps.ctf[idx].contiguous(),
                        ps.sigRcp[idx].contiguous(), qs.contiguous(), ts.contiguous(), pwR, pwT,
                        pwC, cls_all[idx].contiguous(), wC, wR, wT, b, None, precision)
        ctx.sync()
        ar = torch.arange(m, device=dev)
        q_new[s:e] = qs[ar, wR.argmax(1)]
        t_new[s:e] = ts[ar, wT.argmax(1)]
        base[s:e] = b
    return q_new, t_new, base


def plain_method_poses(ctx, ps, quats_g, mats_g, trans_g, precision, gen,
                       schedule=CONVERGE_SCHEDULE):
    """The plain method run to convergence on ps: the global search, then
    one local phase per (kappa, trans_sd) of `schedule`, each about the
    previous phase's best pose.  Returns host arrays quat [n][4], trans
    [n][2] and the median rotation change (degrees) of every local phase."""
    q, t, _ = global_best(ctx, ps, quats_g, mats_g, trans_g, precision)
    moves = []
    for kappa, tsd in schedule:
        qn, tn, _ = local_refine(ctx, ps, q, t, kappa, tsd, precision, gen)
        moves.append(float(np.median(angle_deg(qn.cpu().numpy(), q.cpu().numpy()))))
        q, t = qn, tn
    return q.cpu().numpy(), t.cpu().numpy(), moves
