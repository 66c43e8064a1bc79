"""Seeded synthetic E-step workloads (host-side input generation).

The reference refines real cryo-EM particle stacks; here every input is made
from a fixed seed so that the CUDA path, the oracle and the benchmark all see
the same numbers:

* a reference map made of isotropic Gaussian blobs, generated directly in
  Fourier space on the padded grid.  The transform of a blob of amplitude A,
  width s (pixels) and centre c is A (2 pi s^2)^(3/2) exp(-2 pi^2 s^2 |f|^2)
  exp(-2 pi i f.c), sampled at f = (x, y, z) / (pf N) cycles per pixel.  This
  stands in for Projector::setProjectee (padding, gridding correction and FFT
  of a real-space map, src/Projector.cpp:123-200), which runs once per
  iteration and is outside the hot path;
* particle images in the selected Fourier pixels: CTF x phase shift x the
  exact central slice of the same analytic transform at the true pose, plus
  white complex Gaussian noise at a stated SNR (signal power over noise power
  over the in-cutoff pixels);
* pixel selection restating Optimiser::allocPreCalIdx
  (src/Optimiser.cpp:7942-7992);
* pose hypotheses: HEALPix (ring scheme, Gorski et al. 2005) directions x
  in-plane angles for the global scan, von Mises-Fisher samples on the
  quaternion sphere (Wood 1994) for local rounds, Gaussian translations.

Volumes are returned as complex tensors of shape (vdim, vdim, vdim//2 + 1)
indexed [z, y, x] -- the half-FT storage of Volume::iFTHalf
(include/Image/Volume.h:566-573).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import torch


# --------------------------------------------------------------------------
# pixel selection
# --------------------------------------------------------------------------
def pixel_index(size: int, rU: float, rL: float):
    """Half-plane Fourier pixels with rL <= rint(|k|) < rU and
    rL^2 <= |k|^2 < rU^2, j-outer / i-inner, skipping i == 0 and j < 0
    (Optimiser::allocPreCalIdx, src/Optimiser.cpp:7942-7992).

    Returns int32 arrays iCol, iRow, iSig, iPxl."""
    r = rU + 1
    j = np.arange(int(-r), math.ceil(r) + 1)
    j = j[j < r]
    i = np.arange(0, int(math.floor(r)) + 1)
    jj, ii = np.meshgrid(j, i, indexing="ij")
    jj = jj.ravel()
    ii = ii.ravel()
    keep = ~((ii == 0) & (jj < 0))
    u = ii.astype(np.float64) ** 2 + jj.astype(np.float64) ** 2
    keep &= (u < rU * rU) & (u >= rL * rL)
    v = np.rint(np.hypot(ii, jj)).astype(np.int64)
    keep &= (v < rU) & (v >= rL)
    ii, jj, v = ii[keep], jj[keep], v[keep]
    iPxl = np.where(jj >= 0, jj, jj + size) * (size // 2 + 1) + ii
    return (ii.astype(np.int32), jj.astype(np.int32), v.astype(np.int32),
            iPxl.astype(np.int32))


# --------------------------------------------------------------------------
# rotations
# --------------------------------------------------------------------------
def quat_to_mat(q: np.ndarray) -> np.ndarray:
    """Row-major rotation matrices of unit quaternions (w, x, y, z):
    R = I + 2 w A + 2 A^2 (rotate3D, src/Geometry/Euler.cpp:181-189)."""
    q = np.asarray(q, dtype=np.float64).reshape(-1, 4)
    w, x, y, z = q.T
    A = np.zeros((len(q), 3, 3))
    A[:, 0, 1], A[:, 0, 2] = -z, y
    A[:, 1, 0], A[:, 1, 2] = z, -x
    A[:, 2, 0], A[:, 2, 1] = -y, x
    eye = np.broadcast_to(np.eye(3), A.shape)
    return eye + 2 * w[:, None, None] * A + 2 * A @ A


def quat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Hamilton product of quaternion arrays (..., 4)."""
    aw, ax, ay, az = np.moveaxis(a, -1, 0)
    bw, bx, by, bz = np.moveaxis(b, -1, 0)
    return np.stack([aw * bw - ax * bx - ay * by - az * bz,
                     aw * bx + ax * bw + ay * bz - az * by,
                     aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw], axis=-1)


def haar_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Haar-uniform rotations: normalised 4-D Gaussian vectors, w >= 0."""
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    return q


def euler_zyz_to_quat(phi, theta, psi) -> np.ndarray:
    """Quaternion of R = Rz(phi) Ry(theta) Rz(psi)."""
    def qz(a):
        return np.stack([np.cos(a / 2), 0 * a, 0 * a, np.sin(a / 2)], -1)

    def qy(a):
        return np.stack([np.cos(a / 2), 0 * a, np.sin(a / 2), 0 * a], -1)
    q = quat_mul(quat_mul(qz(phi), qy(theta)), qz(psi))
    q[q[..., 0] < 0] *= -1
    return q


def healpix_ring_centres(nside: int):
    """(theta, phi) of the 12 nside^2 HEALPix pixel centres, ring scheme
    (Gorski et al. 2005, ApJ 622:759, eqs. 4-9)."""
    npix = 12 * nside * nside
    ncap = 2 * nside * (nside - 1)
    out = np.zeros((npix, 2))
    for p in range(npix):
        if p < ncap:                                   # north polar cap
            i = int((1 + math.isqrt(1 + 2 * p)) // 2)
            while 2 * i * (i + 1) <= p:
                i += 1
            while 2 * i * (i - 1) > p:
                i -= 1
            j = p - 2 * i * (i - 1) + 1
            z = 1 - i * i / (3.0 * nside * nside)
            ph = (j - 0.5) * math.pi / (2 * i)
        elif p < npix - ncap:                          # equatorial belt
            pp = p - ncap
            i = pp // (4 * nside) + nside
            j = pp % (4 * nside) + 1
            s = (i - nside + 1) % 2
            z = (2 * nside - i) * 2.0 / (3 * nside)
            ph = (j - s / 2.0) * math.pi / (2 * nside)
        else:                                          # south polar cap
            pp = npix - p - 1
            i = int((1 + math.isqrt(1 + 2 * pp)) // 2)
            while 2 * i * (i + 1) <= pp:
                i += 1
            while 2 * i * (i - 1) > pp:
                i -= 1
            j = 4 * i - (pp - 2 * i * (i - 1))
            z = -(1 - i * i / (3.0 * nside * nside))
            ph = (j - 0.5) * math.pi / (2 * i)
        out[p] = (math.acos(max(-1.0, min(1.0, z))), ph)
    return out


def global_rotations(nside: int = 4, n_psi: int = 36) -> np.ndarray:
    """HEALPix directions x uniform in-plane angles as quaternions
    (192 x 36 = 6,912 for nside 4)."""
    tp = healpix_ring_centres(nside)
    psi = np.arange(n_psi) * (2 * math.pi / n_psi)
    th = np.repeat(tp[:, 0], n_psi)
    ph = np.repeat(tp[:, 1], n_psi)
    ps = np.tile(psi, len(tp))
    return euler_zyz_to_quat(ph, th, ps)


def vmf_quaternions(rng: np.random.Generator, mean: np.ndarray, kappa: float,
                    n: int) -> np.ndarray:
    """n samples of the von Mises-Fisher distribution on S^3 with mean
    direction `mean` and concentration kappa (Wood 1994, Commun. Stat.
    Simul. Comput. 23:157)."""
    p = 4
    b = (-2 * kappa + math.sqrt(4 * kappa * kappa + (p - 1) ** 2)) / (p - 1)
    x0 = (1 - b) / (1 + b)
    c = kappa * x0 + (p - 1) * math.log(1 - x0 * x0)
    w = np.empty(n)
    filled = 0
    while filled < n:
        m = (n - filled) * 2 + 8
        z = rng.beta((p - 1) / 2, (p - 1) / 2, m)
        u = rng.random(m)
        ww = (1 - (1 + b) * z) / (1 - (1 - b) * z)
        ok = kappa * ww + (p - 1) * np.log(1 - x0 * ww) - c >= np.log(u)
        take = ww[ok][: n - filled]
        w[filled:filled + len(take)] = take
        filled += len(take)
    v = rng.standard_normal((n, p - 1))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    samp = np.concatenate([w[:, None], np.sqrt(1 - w * w)[:, None] * v], 1)
    # rotate e0 = (1, 0, 0, 0) onto the mean: left-multiply by the mean
    out = quat_mul(np.broadcast_to(mean, samp.shape), samp)
    out /= np.linalg.norm(out, axis=1, keepdims=True)
    return out


# --------------------------------------------------------------------------
# maps
# --------------------------------------------------------------------------
@dataclass
class BlobMap:
    amp: np.ndarray       # (nb,)
    sigma: np.ndarray     # (nb,) pixels
    centre: np.ndarray    # (nb, 3) pixels, relative to the box centre


def blob_map(rng: np.random.Generator, n_blobs: int, sigma_a: tuple,
             pixel_size: float, radius_px: float) -> BlobMap:
    """n_blobs isotropic Gaussians: widths U(sigma_a) in Angstrom, centres
    uniform in a ball of radius_px pixels, amplitudes U(0.5, 1)."""
    d = rng.standard_normal((n_blobs, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rad = radius_px * rng.random(n_blobs) ** (1.0 / 3.0)
    return BlobMap(amp=rng.uniform(0.5, 1.0, n_blobs),
                   sigma=rng.uniform(*sigma_a, n_blobs) / pixel_size,
                   centre=d * rad[:, None])


def class_maps(rng: np.random.Generator, n_classes: int, shared: float, n_blobs: int,
               sigma_a: tuple, pixel_size: float, radius_px: float) -> list:
    """n_classes blob maps sharing a fraction `shared` of their n_blobs
    blobs: one base map whose remaining blobs (one fixed index set) are
    re-drawn for every class.  One class returns the base map itself."""
    base = blob_map(rng, n_blobs, sigma_a, pixel_size, radius_px)
    if n_classes == 1:
        return [base]
    n_new = int(round(n_blobs * (1.0 - shared)))
    idx = rng.choice(n_blobs, n_new, replace=False)
    maps = []
    for _ in range(n_classes):
        fresh = blob_map(rng, n_new, sigma_a, pixel_size, radius_px)
        amp, sig, cen = base.amp.copy(), base.sigma.copy(), base.centre.copy()
        amp[idx], sig[idx], cen[idx] = fresh.amp, fresh.sigma, fresh.centre
        maps.append(BlobMap(amp=amp, sigma=sig, centre=cen))
    return maps


def blob_ft(bm: BlobMap, f: torch.Tensor) -> torch.Tensor:
    """Analytic Fourier transform of the blob map at frequencies f (..., 3)
    in cycles per pixel."""
    dt = f.dtype
    amp = torch.as_tensor(bm.amp, dtype=dt, device=f.device)
    s2 = torch.as_tensor(bm.sigma ** 2, dtype=dt, device=f.device)
    c = torch.as_tensor(bm.centre, dtype=dt, device=f.device)
    f2 = (f * f).sum(-1, keepdim=True)                       # (..., 1)
    env = amp * (2 * math.pi * s2) ** 1.5 * torch.exp(-2 * math.pi ** 2 * s2 * f2)
    ph = -2 * math.pi * (f @ c.T)                             # (..., nb)
    re = (env * torch.cos(ph)).sum(-1)
    im = (env * torch.sin(ph)).sum(-1)
    return torch.complex(re, im)


def padded_volume(bm: BlobMap, box: int, pf: int, device="cpu",
                  dtype=torch.float64, chunk: int = 1 << 21) -> torch.Tensor:
    """The map's transform on the padded half-FT grid: complex tensor
    (vdim, vdim, vdim//2 + 1), vdim = pf * box, indexed [z, y, x]."""
    vdim = pf * box
    nx = vdim // 2 + 1
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    out = torch.empty((vdim, vdim, nx), dtype=cdt, device=device)
    flat = out.view(-1)
    n = flat.numel()
    idx_all = torch.arange(n, device=device)
    for s in range(0, n, chunk):
        idx = idx_all[s:s + chunk]
        x = idx % nx
        y = (idx // nx) % vdim
        z = idx // (nx * vdim)
        y = torch.where(y < vdim // 2, y, y - vdim)
        z = torch.where(z < vdim // 2, z, z - vdim)
        f = torch.stack([x, y, z], -1).to(dtype) / vdim
        flat[s:s + chunk] = blob_ft(bm, f)
    return out


def class_images_2d(maps, box: int, pf: int, device="cpu") -> torch.Tensor:
    """2-D class images: the transform of each map's projection along z (its
    central section) on the padded half grid, complex64 (nK, vdim, vdim//2 + 1),
    indexed [k, y, x]."""
    vdim = pf * box
    nx = vdim // 2 + 1
    y = torch.arange(vdim, device=device)
    y = torch.where(y < vdim // 2, y, y - vdim).to(torch.float64)
    x = torch.arange(nx, device=device, dtype=torch.float64)
    f = torch.stack([x[None, :].expand(vdim, nx), y[:, None].expand(vdim, nx),
                     torch.zeros(vdim, nx, dtype=torch.float64, device=device)], -1) / vdim
    return torch.stack([blob_ft(bm, f) for bm in maps]).to(torch.complex64)


def sample_2d(imgs: torch.Tensor, k: torch.Tensor, rot: torch.Tensor, iCol, iRow, pf: int):
    """Bilinear samples of class images imgs (nK, vdim, nx) at the in-plane
    rotations rot (n, 2) = (cos, sin) of the padded pixels (iCol pf, iRow pf),
    class k (n,) per row; a point with x < 0 reads (-x, -y) conjugated and
    rows wrap: (n, K) complex64."""
    nK, vdim, nx = imgs.shape
    dev = imgs.device
    a = torch.as_tensor(np.asarray(iCol) * pf, dtype=torch.float32, device=dev)[None, :]
    b = torch.as_tensor(np.asarray(iRow) * pf, dtype=torch.float32, device=dev)[None, :]
    c, s = rot[:, 0:1].float(), rot[:, 1:2].float()
    x, y = c * a - s * b, s * a + c * b
    neg = x < 0
    x, y = torch.where(neg, -x, x), torch.where(neg, -y, y)
    x0, y0 = torch.floor(x), torch.floor(y)
    fx, fy = x - x0, y - y0
    x0, y0 = x0.long(), y0.long()
    flat = imgs.reshape(nK, -1)
    out = torch.zeros(x.shape, dtype=torch.complex64, device=dev)
    for j in (0, 1):
        yy = torch.remainder(y0 + j, vdim)
        wy = fy if j else 1 - fy
        for i in (0, 1):
            wx = fx if i else 1 - fx
            v = flat[k[:, None], yy * nx + x0 + i]
            out = out + v * (wx * wy)
    return torch.where(neg, out.conj(), out)


# --------------------------------------------------------------------------
# CTF
# --------------------------------------------------------------------------
CTF_FIELDS = ("voltage", "defocusU", "defocusV", "defocusTheta", "Cs",
              "amplitudeContrast", "phaseShift")


def ctf_attrs(rng: np.random.Generator, n: int, voltage_kv=300.0, cs_mm=2.7,
              amp=0.1, defocus_um=(1.0, 3.0)) -> np.ndarray:
    """(n, 7) float64 rows in CTFAttr field order (include/Database.h:108-122),
    in the units CTF() expects: volts, Angstrom, radians."""
    a = np.zeros((n, 7))
    a[:, 0] = voltage_kv * 1e3
    a[:, 1] = rng.uniform(*defocus_um, n) * 1e4
    a[:, 2] = rng.uniform(*defocus_um, n) * 1e4
    a[:, 3] = rng.uniform(0, math.pi, n)
    a[:, 4] = cs_mm * 1e7
    a[:, 5] = amp
    a[:, 6] = 0.0
    return a


def ctf_values(attr: np.ndarray, pixel_size: float, N: int, iCol, iRow):
    """CTF at the selected pixels for every row of attr (vectorised form of
    CTF(RFLOAT*, ...), src/CTF.cpp:98-145); (n, K) float64."""
    attr = np.atleast_2d(attr)
    V, dU, dV, th, Cs, A, ps = [attr[:, k:k + 1] for k in range(7)]
    lam = 12.2643247 / np.sqrt(V * (1 + V * 0.978466e-6))
    K1 = math.pi * lam
    K2 = (math.pi / 2) * Cs * lam ** 3
    u = np.hypot(iCol / (pixel_size * N), iRow / (pixel_size * N))[None, :]
    ang = np.arctan2(iRow, iCol)[None, :] - th
    dfc = -(dU + dV + (dU - dV) * np.cos(2 * ang)) / 2
    ki = K1 * dfc * u ** 2 + K2 * u ** 4 - ps
    return -np.sqrt(1 - A * A) * np.sin(ki) + A * np.cos(ki)


def phase_shift(trans: np.ndarray, N: int, iCol, iRow) -> np.ndarray:
    """exp(-2 pi i (iCol tx + iRow ty) / N) for each translation: (nT, K)."""
    trans = np.atleast_2d(trans)
    ph = 2 * math.pi * (np.outer(trans[:, 0] / N, iCol) + np.outer(trans[:, 1] / N, iRow))
    return np.exp(-1j * ph)


# --------------------------------------------------------------------------
# a particle stack
# --------------------------------------------------------------------------
@dataclass
class Stack:
    box: int
    pixel_size: float
    pf: int
    rU: float
    rL: float
    iCol: np.ndarray
    iRow: np.ndarray
    iSig: np.ndarray
    quat_true: np.ndarray       # (n, 4)
    trans_true: np.ndarray      # (n, 2) pixels
    ctf_attr: np.ndarray        # (n, 7)
    ctf: np.ndarray             # (n, K) float64
    dat: np.ndarray             # (n, K) complex128
    sigRcp: np.ndarray          # (n, K) float64, -1 / (2 s^2)
    noise_s2: float
    maps: list = field(default_factory=list)
    cls_true: np.ndarray = None

    @property
    def K(self):
        return len(self.iCol)


def make_stack(seed: int, maps, box: int, pixel_size: float, pf: int,
               rU: float, rL: float, n: int, shift_range: float, snr: float,
               device="cpu") -> Stack:
    """n particles from `maps` (assigned round-robin, 1:1:...) at Haar-uniform
    poses and U(-shift_range, shift_range) shifts, with white noise at `snr`."""
    rng = np.random.default_rng(seed)
    iCol, iRow, iSig, _ = pixel_index(box, rU, rL)
    K = len(iCol)
    q = haar_quaternions(rng, n)
    t = rng.uniform(-shift_range, shift_range, (n, 2))
    attr = ctf_attrs(rng, n)
    ctf = ctf_values(attr, pixel_size, box, iCol, iRow)
    cls = np.arange(n) % len(maps)
    R = quat_to_mat(q)
    k2 = np.stack([iCol, iRow, np.zeros(K)], 0).astype(np.float64) / box  # (3, K)
    sig = np.zeros((n, K), dtype=np.complex128)
    for c, bm in enumerate(maps):
        sel = np.nonzero(cls == c)[0]
        step = max(1, (1 << 27) // max(1, K * len(bm.amp)))   # bound the (n, K, blobs) temporaries
        for s in range(0, len(sel), step):
            ids = sel[s:s + step]
            f = torch.as_tensor(np.einsum("nij,jk->nki", R[ids], k2), device=device)
            sig[ids] = blob_ft(bm, f).cpu().numpy()
    sig = sig * ctf * np.exp(-2j * math.pi * (np.outer(t[:, 0] / box, iCol)
                                              + np.outer(t[:, 1] / box, iRow)))
    p_sig = float(np.mean(np.abs(sig) ** 2))
    s2 = p_sig / snr / 2.0
    noise = rng.standard_normal((n, K)) + 1j * rng.standard_normal((n, K))
    dat = sig + math.sqrt(s2) * noise
    sigRcp = np.full((n, K), -1.0 / (2.0 * s2))
    return Stack(box=box, pixel_size=pixel_size, pf=pf, rU=rU, rL=rL,
                 iCol=iCol, iRow=iRow, iSig=iSig, quat_true=q, trans_true=t,
                 ctf_attr=attr, ctf=ctf, dat=dat, sigRcp=sigRcp, noise_s2=s2,
                 maps=list(maps), cls_true=cls)


# --------------------------------------------------------------------------
# named workloads
# --------------------------------------------------------------------------
@dataclass
class ParticleSet:
    images: torch.Tensor       # (n, img, img) float32, per-image normalised (device)
    dat: np.ndarray            # (n, K) complex64: the same data at the cutoff's pixels
    ctf: np.ndarray            # (n, K) float32
    sigRcp: np.ndarray         # (n, K) float32
    iCol: np.ndarray
    iRow: np.ndarray
    quat_true: np.ndarray      # (n, 4)
    trans_true: np.ndarray     # (n, 2) pixels at the full box
    cls: np.ndarray            # (n,) map of every particle


def particle_set(seed: int, maps, cls, box: int, pixel_size: float, rU: float, rL: float,
                 shift_range: float, snr: float, img: int = 64, device="cpu",
                 chunk: int = 512, noise_var: float | None = None,
                 with_data: bool = True) -> ParticleSet:
    """Particles of several maps (particle l shows maps[cls[l]]) at Haar-uniform
    poses and U(-shift_range, shift_range) shifts, with CTF and white noise at
    `snr` (signal / noise power over the band-limited image grid), or of
    variance `noise_var` per real and imaginary part when given.

    The data of a particle is one noisy transform on the union of two pixel
    sets at the full box's frequencies: the rfft grid of an img x img image
    (|k| <= img / 2, i.e. the box band-limited and downsampled by box / img)
    and the pixels of cutoff rU (the likelihood's input).  Its real-space image
    (the network's input, centred, normalised to zero mean and unit
    deviation) and its values at the likelihood's pixels come from that one
    transform, so both see the same particle.  with_data=False computes the
    image only (dat, ctf and sigRcp are then empty)."""
    rng = np.random.default_rng(seed)
    cls = np.asarray(cls)
    n = len(cls)
    q = haar_quaternions(rng, n)
    t = rng.uniform(-shift_range, shift_range, (n, 2))
    attr = ctf_attrs(rng, n)
    h = img // 2
    jj = np.concatenate([np.arange(0, h), np.arange(-h, 0)])     # FFT row order
    ii = np.arange(0, h + 1)
    J, I = np.meshgrid(jj, ii, indexing="ij")
    gi, gj = I.ravel(), J.ravel()                                  # image grid (img (h + 1),)
    iCol, iRow, _, _ = pixel_index(box, rU, rL)
    if with_data:
        # union of the image grid and the likelihood's pixels, image grid first
        key_img = gj.astype(np.int64) * (box + 1) + gi
        key_lik = iRow.astype(np.int64) * (box + 1) + iCol
        img_pos = {int(k): i for i, k in enumerate(key_img)}
        inside = np.isin(key_lik, key_img)
        ui = np.concatenate([gi, iCol[~inside]])
        uj = np.concatenate([gj, iRow[~inside]])
        lik = np.empty(len(iCol), np.int64)
        lik[inside] = [img_pos[int(k)] for k in key_lik[inside]]
        lik[~inside] = len(gi) + np.arange(int((~inside).sum()))
    else:
        ui, uj, lik = gi, gj, None
    G = len(gi)
    ctf_u = ctf_values(attr, pixel_size, box, ui, uj)              # (n, U)
    R = quat_to_mat(q)
    k2 = np.stack([ui, uj, np.zeros_like(ui)], 0).astype(np.float32) / box
    sig = np.empty((n, len(ui)), np.complex64)
    for c in range(len(maps)):
        sel_c = np.nonzero(cls == c)[0]
        for s0 in range(0, len(sel_c), chunk):
            ids = sel_c[s0:s0 + chunk]
            f = torch.as_tensor(np.einsum("nij,jk->nki", R[ids].astype(np.float32), k2), device=device)
            sig[ids] = blob_ft(maps[c], f).cpu().numpy()
    sig *= ctf_u.astype(np.float32)
    sig *= np.exp(-2j * math.pi * (np.outer(t[:, 0] / box, ui) + np.outer(t[:, 1] / box, uj))).astype(np.complex64)
    if noise_var is None:
        p_sig = float(np.mean(np.abs(sig[:, :G]) ** 2))
        s2 = p_sig / snr / 2.0
    else:
        s2 = float(noise_var)
    noise = (rng.standard_normal(sig.shape) + 1j * rng.standard_normal(sig.shape)) * math.sqrt(s2)
    data = (sig + noise.astype(np.complex64)).astype(np.complex64)
    grid = torch.as_tensor(np.ascontiguousarray(data[:, :G]).reshape(n, img, h + 1), device=device)
    ims = torch.fft.irfft2(grid, s=(img, img))
    ims = torch.fft.fftshift(ims, dim=(-2, -1))
    ims = ims - ims.mean(dim=(-2, -1), keepdim=True)
    ims = ims / ims.std(dim=(-2, -1), keepdim=True)
    if with_data:
        dat = np.ascontiguousarray(data[:, lik])
        ctf_k = np.ascontiguousarray(ctf_u[:, lik].astype(np.float32))
        sigr = np.full((n, len(iCol)), -1.0 / (2.0 * s2), np.float32)
    else:
        dat = np.zeros((n, 0), np.complex64)
        ctf_k = np.zeros((n, 0), np.float32)
        sigr = np.zeros((n, 0), np.float32)
    return ParticleSet(images=ims.float().contiguous(), dat=dat, ctf=ctf_k, sigRcp=sigr,
                       iCol=iCol, iRow=iRow, quat_true=q, trans_true=t, cls=cls)


def signal_power(maps, box: int, pixel_size: float, rU: float, rL: float, n: int = 64,
                 seed: int = 0, device="cpu") -> float:
    """Mean |signal|^2 (CTF applied) over the pixels of cutoff rU of n
    particles of every map: the noise variance of an SNR defined over the
    likelihood's pixels is this / snr / 2 per real and imaginary part."""
    rng = np.random.default_rng(seed)
    iCol, iRow, _, _ = pixel_index(box, rU, rL)
    k2 = np.stack([iCol, iRow, np.zeros_like(iCol)], 0).astype(np.float32) / box
    tot = 0.0
    for bm in maps:
        q = haar_quaternions(rng, n)
        attr = ctf_attrs(rng, n)
        ctf_k = ctf_values(attr, pixel_size, box, iCol, iRow)
        f = torch.as_tensor(np.einsum("nij,jk->nki", quat_to_mat(q).astype(np.float32), k2),
                            device=device)
        s = blob_ft(bm, f).cpu().numpy() * ctf_k
        tot += float(np.mean(np.abs(s) ** 2))
    return tot / len(maps)


def global_translations(half: int = 3, step: float = 1.0) -> np.ndarray:
    """(2 half + 1)^2 grid of shifts, `step` pixels apart (7 x 7 = 49)."""
    g = np.arange(-half, half + 1) * step
    tx, ty = np.meshgrid(g, g, indexing="ij")
    return np.stack([tx.ravel(), ty.ravel()], 1)


def vmf_quaternions_many(rng: np.random.Generator, means: np.ndarray, kappa: float,
                         counts) -> np.ndarray:
    """counts[i] vMF samples about means[i] (one concentration for all), as
    vmf_quaternions draws them, packed particle after particle:
    (sum(counts), 4)."""
    counts = np.asarray(counts, dtype=np.int64)
    n = int(counts.sum())
    p = 4
    b = (-2 * kappa + math.sqrt(4 * kappa * kappa + (p - 1) ** 2)) / (p - 1)
    x0 = (1 - b) / (1 + b)
    c = kappa * x0 + (p - 1) * math.log(1 - x0 * x0)
    w = np.empty(n)
    filled = 0
    while filled < n:
        m = (n - filled) * 2 + 8
        z = rng.beta((p - 1) / 2, (p - 1) / 2, m)
        u = rng.random(m)
        ww = (1 - (1 + b) * z) / (1 - (1 - b) * z)
        ok = kappa * ww + (p - 1) * np.log(1 - x0 * ww) - c >= np.log(u)
        take = ww[ok][: n - filled]
        w[filled:filled + len(take)] = take
        filled += len(take)
    v = rng.standard_normal((n, p - 1))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    samp = np.concatenate([w[:, None], np.sqrt(1 - w * w)[:, None] * v], 1)
    out = quat_mul(np.repeat(means, counts, axis=0), samp)
    out /= np.linalg.norm(out, axis=1, keepdims=True)
    return out


def local_hypotheses(rng: np.random.Generator, q_centre: np.ndarray,
                     t_centre: np.ndarray, nR: int, nT: int, kappa: float,
                     trans_sd: float):
    """Per-particle local hypothesis sets: nR vMF rotations about q_centre
    and nT Gaussian translations about t_centre.  Returns (n, nR, 4) and
    (n, nT, 2) float64."""
    n = len(q_centre)
    qs = np.empty((n, nR, 4))
    for i in range(n):
        qs[i] = vmf_quaternions(rng, q_centre[i], kappa, nR)
    ts = t_centre[:, None, :] + trans_sd * rng.standard_normal((n, nT, 2))
    return qs, ts


def perturb_poses(rng: np.random.Generator, q: np.ndarray, t: np.ndarray,
                  rot_deg: float, trans_px: float):
    """Current poses a small random step away from the true ones."""
    axis = rng.standard_normal((len(q), 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    ang = np.deg2rad(rot_deg) * rng.random(len(q))
    dq = np.concatenate([np.cos(ang / 2)[:, None], np.sin(ang / 2)[:, None] * axis], 1)
    qn = quat_mul(q, dq)
    qn /= np.linalg.norm(qn, axis=1, keepdims=True)
    return qn, t + trans_px * rng.standard_normal(t.shape)


CONFIGS = {
    # configuration 0: 64^3, global scan, CPU-runnable
    "box64_global": dict(box=64, pixel_size=1.5, n_blobs=40, sigma_a=(2.0, 4.0),
                         radius_px=20.0, n=2000, shift=3.0, snr=0.05, rU=16,
                         pf=2, n_classes=1),
    # configuration 1: 256^3, local rounds 1,000 rotations x 100 translations
    "box256_local": dict(box=256, pixel_size=1.1, n_blobs=200, sigma_a=(1.5, 3.0),
                         radius_px=80.0, n=50000, shift=8.0, snr=0.03, rU=80,
                         pf=2, n_classes=1, nR=1000, nT=100, kappa=200.0),
}


def config_rL(box: int, pixel_size: float, ignore_res: float = 200.0) -> float:
    """Lower pixel radius of the likelihood,
    rL = floor(resA2P(1 / ignoreRes, size, pixelSize)) (src/Optimiser.cpp:243,
    resA2P src/Functions/Spectrum.cpp:26-31); ignoreRes 200 Angstrom."""
    return float(math.floor(box * pixel_size / ignore_res))


# --------------------------------------------------------------------------
# device-side generators (large particle sets: training sets at box 256)
# --------------------------------------------------------------------------
def quat_mul_t(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """Hamilton product of quaternion tensors (..., 4)."""
    aw, ax, ay, az = a.unbind(-1)
    bw, bx, by, bz = b.unbind(-1)
    return torch.stack([aw * bw - ax * bx - ay * by - az * bz,
                        aw * bx + ax * bw + ay * bz - az * by,
                        aw * by - ax * bz + ay * bw + az * bx,
                        aw * bz + ax * by - ay * bx + az * bw], dim=-1)


def vmf_quaternions_dev(gen: torch.Generator, means: torch.Tensor, kappa: float,
                        n: int) -> torch.Tensor:
    """n von Mises-Fisher samples about each of means [m][4] (float64,
    device) with concentration kappa: [m][n][4] float64.  Wood's (1994)
    rejection sampler, as vmf_quaternions; its Beta((p-1)/2, (p-1)/2) proposal
    for p = 4 is drawn as (1 + g0 / |g|) / 2 with g a standard 4-D Gaussian
    (the first coordinate of a uniform point of S^3), and the samples are
    drawn with the device generator `gen`."""
    dev = means.device
    m = means.shape[0]
    p = 4
    b = (-2 * kappa + math.sqrt(4 * kappa * kappa + (p - 1) ** 2)) / (p - 1)
    x0 = (1 - b) / (1 + b)
    c = kappa * x0 + (p - 1) * math.log(1 - x0 * x0)
    total = m * n
    w = torch.empty(total, dtype=torch.float64, device=dev)
    filled = 0
    while filled < total:
        k = int((total - filled) * 1.3) + 64
        g = torch.randn((k, 4), generator=gen, dtype=torch.float64, device=dev)
        z = 0.5 * (1.0 + g[:, 0] / g.norm(dim=1))
        u = torch.rand(k, generator=gen, dtype=torch.float64, device=dev)
        ww = (1 - (1 + b) * z) / (1 - (1 - b) * z)
        ok = kappa * ww + (p - 1) * torch.log(1 - x0 * ww) - c >= torch.log(u)
        take = ww[ok][: total - filled]
        w[filled:filled + take.numel()] = take
        filled += take.numel()
    v = torch.randn((total, 3), generator=gen, dtype=torch.float64, device=dev)
    v = v / v.norm(dim=1, keepdim=True)
    samp = torch.cat([w[:, None], torch.sqrt(torch.clamp(1 - w * w, min=0.0))[:, None] * v], 1)
    out = quat_mul_t(means.to(torch.float64).repeat_interleave(n, 0), samp)
    out = out / out.norm(dim=1, keepdim=True)
    return out.view(m, n, 4)


def local_hypotheses_dev(gen: torch.Generator, q_centre: torch.Tensor, t_centre: torch.Tensor,
                         nR: int, nT: int, kappa: float, trans_sd: float):
    """local_hypotheses on the device: nR vMF rotations about each q_centre
    [m][4] and nT Gaussian translations (deviation trans_sd) about each
    t_centre [m][2]; float64 tensors [m][nR][4] and [m][nT][2]."""
    qs = vmf_quaternions_dev(gen, q_centre, kappa, nR)
    ts = t_centre.to(torch.float64)[:, None, :] + trans_sd * torch.randn(
        (q_centre.shape[0], nT, 2), generator=gen, dtype=torch.float64, device=q_centre.device)
    return qs, ts


def ctf_values_t(attr: torch.Tensor, pixel_size: float, N: int, iCol: torch.Tensor,
                 iRow: torch.Tensor) -> torch.Tensor:
    """ctf_values on tensors (float64): attr [n][7], pixels iCol / iRow [K]."""
    V, dU, dV, th, Cs, A, ps = [attr[:, k:k + 1] for k in range(7)]
    lam = 12.2643247 / torch.sqrt(V * (1 + V * 0.978466e-6))
    K1 = math.pi * lam
    K2 = (math.pi / 2) * Cs * lam ** 3
    fc = iCol.to(torch.float64) / (pixel_size * N)
    fr = iRow.to(torch.float64) / (pixel_size * N)
    u = torch.hypot(fc, fr)[None, :]
    ang = torch.atan2(iRow.to(torch.float64), iCol.to(torch.float64))[None, :] - th
    dfc = -(dU + dV + (dU - dV) * torch.cos(2 * ang)) / 2
    ki = K1 * dfc * u ** 2 + K2 * u ** 4 - ps
    return -torch.sqrt(1 - A * A) * torch.sin(ki) + A * torch.cos(ki)


@dataclass
class ParticleSetDev:
    images: torch.Tensor       # (n, img, img) float32, per-image normalised
    dat: torch.Tensor          # (n, K) complex64 at the likelihood's pixels
    ctf: torch.Tensor          # (n, K) float32
    sigRcp: torch.Tensor       # (n, K) float32
    iCol: np.ndarray
    iRow: np.ndarray
    quat_true: np.ndarray      # (n, 4)
    trans_true: np.ndarray     # (n, 2)
    cls: np.ndarray            # (n,)


def particle_set_dev(seed: int, maps, cls, box: int, pixel_size: float, rU: float, rL: float,
                     shift_range: float, noise_var: float, img: int = 64, device="cuda",
                     chunk: int = 2048) -> ParticleSetDev:
    """particle_set with every per-pixel array made and kept on the device:
    the same model (one noisy transform on the union of the img x img image
    grid and the likelihood's pixels, CTF, phase shift, white noise of
    variance noise_var per part) with poses and CTF parameters from a numpy
    generator seeded `seed` and the noise from a device generator seeded
    `seed`."""
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed))
    cls = np.asarray(cls)
    n = len(cls)
    q = haar_quaternions(rng, n)
    t = rng.uniform(-shift_range, shift_range, (n, 2))
    attr = ctf_attrs(rng, n)
    h = img // 2
    jj = np.concatenate([np.arange(0, h), np.arange(-h, 0)])
    ii = np.arange(0, h + 1)
    J, I = np.meshgrid(jj, ii, indexing="ij")
    gi, gj = I.ravel(), J.ravel()
    iCol, iRow, _, _ = pixel_index(box, rU, rL)
    key_img = gj.astype(np.int64) * (box + 1) + gi
    key_lik = iRow.astype(np.int64) * (box + 1) + iCol
    img_pos = {int(k): i for i, k in enumerate(key_img)}
    inside = np.isin(key_lik, key_img)
    ui = np.concatenate([gi, iCol[~inside]])
    uj = np.concatenate([gj, iRow[~inside]])
    lik = np.empty(len(iCol), np.int64)
    lik[inside] = [img_pos[int(k)] for k in key_lik[inside]]
    lik[~inside] = len(gi) + np.arange(int((~inside).sum()))
    G, K = len(gi), len(iCol)
    ui_t = torch.as_tensor(ui, device=device)
    uj_t = torch.as_tensor(uj, device=device)
    lik_t = torch.as_tensor(lik, device=device)
    k2 = torch.stack([ui_t, uj_t, torch.zeros_like(ui_t)], 0).to(torch.float32) / box
    R = torch.as_tensor(quat_to_mat(q).astype(np.float32), device=device)
    attr_t = torch.as_tensor(attr, device=device)
    tt = torch.as_tensor(t, device=device)
    images = torch.empty((n, img, img), dtype=torch.float32, device=device)
    dat = torch.empty((n, K), dtype=torch.complex64, device=device)
    ctf_k = torch.empty((n, K), dtype=torch.float32, device=device)
    sd = math.sqrt(noise_var)
    for s0 in range(0, n, chunk):
        s1 = min(n, s0 + chunk)
        idx = np.arange(s0, s1)
        sig = torch.empty((s1 - s0, len(ui)), dtype=torch.complex64, device=device)
        for c in np.unique(cls[idx]):
            sel = np.nonzero(cls[idx] == c)[0]
            sel_t = torch.as_tensor(sel, device=device)
            f = torch.einsum("nij,jk->nki", R[s0 + sel_t], k2)
            sig[sel_t] = blob_ft(maps[int(c)], f)
        ctf_u = ctf_values_t(attr_t[s0:s1], pixel_size, box, ui_t, uj_t)
        ph = -2 * math.pi * (tt[s0:s1, 0:1] / box * ui_t[None, :].to(torch.float64)
                             + tt[s0:s1, 1:2] / box * uj_t[None, :].to(torch.float64))
        sig = sig * (ctf_u * torch.exp(1j * ph)).to(torch.complex64)
        noise = torch.complex(torch.randn(sig.shape, generator=gen, device=device),
                              torch.randn(sig.shape, generator=gen, device=device)) * sd
        data = sig + noise
        grid = data[:, :G].reshape(s1 - s0, img, h + 1)
        ims = torch.fft.irfft2(grid, s=(img, img))
        ims = torch.fft.fftshift(ims, dim=(-2, -1))
        ims = ims - ims.mean(dim=(-2, -1), keepdim=True)
        images[s0:s1] = (ims / ims.std(dim=(-2, -1), keepdim=True)).float()
        dat[s0:s1] = data[:, lik_t]
        ctf_k[s0:s1] = ctf_u[:, lik_t].float()
    sigRcp = torch.full((n, K), -1.0 / (2.0 * noise_var), dtype=torch.float32, device=device)
    return ParticleSetDev(images=images, dat=dat, ctf=ctf_k, sigRcp=sigRcp, iCol=iCol,
                          iRow=iRow, quat_true=q, trans_true=t, cls=cls)
