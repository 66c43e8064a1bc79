"""Oracle (test infrastructure only): Reconstructor::reconstruct
(src/Reconstructor.cpp:1129-1790; 3-D and 2-D, no symmetry) in numpy float64
-- the checker for tg3_ctx_reconstruct_d and tg3_Reconstruct2D, never on the
product path.  The 2-D mode is the same chain on the padded 2-D half grid
(the reference's _T2D / _W2D / _C2D branches, with the same MKB_RL and TIK_RL
forms at |x| / (pf N)).  The kernel functions use scipy's Bessel functions
(MKB_RL, TIK_RL of src/Functions/Functions.cpp:128-220); the balancing kernel
is looked up at r^2 rounded to the reference's table step.  The transforms
are numpy's (unnormalised forward, 1/n inverse, as the reference's FFTW
wrappers, src/FFT.cpp).  Pinned: the whole chain matches the compiled
reference (with the vendored FFTW) to 1e-12 of the map's peak, live in
tests/test_oracle_pin.py and by the fixtures of tests/golden/ref_golden_recon.npz
in tests/test_oracle_golden.py."""
from __future__ import annotations

import numpy as np
from scipy import special


def mkb_rl(r, a, alpha):
    """Real-space form of the order-0 modified Kaiser-Bessel kernel."""
    r = np.asarray(r, np.float64)
    u = 2 * np.pi * a * r
    w = (2 * np.pi) ** 1.5 * a ** 3 / special.i0(alpha)
    v = np.sqrt(np.abs(alpha * alpha - u * u))
    vs = np.maximum(v, 1e-300)
    inner = np.where(v < 1e-8, 1.0 / (2 ** 1.5 * special.gamma(2.5)), special.iv(1.5, vs) / vs ** 1.5)
    outer = np.where(v < 1e-8, 1.0 / (2 ** 1.5 * special.gamma(2.5)), special.jv(1.5, vs) / vs ** 1.5)
    return w * np.where(u <= alpha, inner, outer)


def tik_rl(r):
    """j0(pi r)^2, the trilinear kernel's real-space form."""
    return np.sinc(np.asarray(r, np.float64)) ** 2


def _coords(vdim, dim=3):
    c = np.fft.fftfreq(vdim, 1.0 / vdim)
    g = np.meshgrid(*([c] * (dim - 1) + [np.arange(vdim // 2 + 1)]), indexing="ij")
    return sum(v * v for v in g)


def reconstruct(F, T, pf, max_radius, fsc=None, join_half=False, grid_corr=True, kernel="trilinear",
                a=1.9, alpha=15.0, kernel_step=1.0 / 100000):
    """F (complex), T (real) on the padded half grid (vdim, vdim, vdim/2 + 1),
    or (vdim, vdim/2 + 1) in 2-D -> the map (N, N, N) or image (N, N)
    centred (coordinate i at index i + N/2) and the number of balancing
    rounds.  The balancing kernel is taken at r^2 rounded to the nearest
    multiple of kernel_step, as the reference's table of it
    (Reconstructor::_kernelRL, a TabFunction of r^2 over [0, 1] in 1e5 steps,
    src/Reconstructor.cpp:76-85, looked up by src/TabFunction.cpp:42-45);
    kernel_step = 0 evaluates it exactly."""
    dim = F.ndim
    vdim = F.shape[0]
    N = vdim // pf
    q = _coords(vdim, dim)
    r2max = (max_radius * pf) ** 2
    inside = q < r2max
    T = np.asarray(T, np.float64).copy()
    if fsc is not None:
        u = np.rint(np.sqrt(q)).astype(int) // pf
        f = np.where(u < len(fsc), np.asarray(fsc)[np.minimum(u, len(fsc) - 1)], 0.0)
        f = np.clip(f, 1e-3, 1 - 1e-3)
        if join_half:
            f = np.sqrt(2 * f / (1 + f))
        sel = (q >= (5 * pf) ** 2) & inside
        T[sel] /= f[sel]
    T = np.maximum(T, 1e-25)
    W = inside.astype(np.float64)
    rounds = 0
    if grid_corr:
        c = np.fft.fftfreq(vdim, 1.0 / vdim)
        g = np.meshgrid(*([c] * dim), indexing="ij")
        r2 = sum(v * v for v in g) / float(N * pf) ** 2
        if kernel_step > 0:
            r2 = np.rint(r2 / kernel_step) * kernel_step
        krl = mkb_rl(np.sqrt(r2), a, alpha) / mkb_rl(0.0, a, alpha)
        diff, no_dec = np.inf, 0
        axes = tuple(range(dim))
        for m in range(30):
            C = np.fft.rfftn(np.fft.irfftn(T * W, s=(vdim,) * dim, axes=axes) * krl, axes=axes)
            mag = np.abs(C)
            W[inside] /= np.maximum(mag[inside], 1e-6)
            prev, diff = diff, np.abs(mag[inside] - 1).max()
            no_dec = no_dec + 1 if diff > prev * 0.95 else 0
            rounds = m + 1
            if diff < 1e-2 or (m >= 10 and no_dec == 2):
                break
    else:
        W[inside] = 1.0 / np.maximum(np.abs(T[inside]), 1e-6)
    V = np.where(inside, F * W, 0)
    pad = np.fft.irfftn(V, s=(vdim,) * dim, axes=tuple(range(dim)))
    idx = np.arange(N) - N // 2
    vol = pad[np.ix_(*([idx % vdim] * dim))]
    g = np.meshgrid(*([idx] * dim), indexing="ij")
    r = np.sqrt(sum(v * v for v in g)) / (pf * N)
    if kernel == "mkb":
        k = mkb_rl(r, a * pf, alpha) / mkb_rl(0.0, a * pf, alpha)
    else:
        k = tik_rl(r)
    return vol / k, rounds
