"""CPU checks of the pose-proposal network's oracle: its analytic gradients
against central finite differences (head, and a reduced network), and its
bf16 rounding."""
import numpy as np

from oracle import cnn_oracle as C

TINY = [(1, 4, 8, 8, 1), (4, 4, 8, 4, 2), (64, 8, 1, 1, 0), (8, 68, 1, 1, 0)]


def _rot(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                     np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                     np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)


def test_head_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    out = rng.standard_normal((3, 68))
    R = _rot(rng, 3)
    t = rng.standard_normal((3, 2))
    loss, g = C.head_loss(out, R, t)
    h = 1e-6
    for i in range(3):
        for j in range(68):
            p, m = out.copy(), out.copy()
            p[i, j] += h
            m[i, j] -= h
            fd = (C.head_loss(p, R, t)[0][i] - C.head_loss(m, R, t)[0][i]) / (2 * h)
            assert abs(fd - g[i, j]) < 1e-5 * max(1.0, abs(fd)), (i, j, fd, g[i, j])


def test_network_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    _, total = C.layout(TINY)
    params = (0.3 * rng.standard_normal(total)).astype(np.float32)
    img = rng.standard_normal((2, 8, 8))
    R = _rot(rng, 2)
    t = rng.standard_normal((2, 2))
    loss, grad = C.loss_and_grad(params, img, R, t, TINY, round_bf16=False)
    h = 1e-3
    for i in rng.choice(total, 60, replace=False):
        p = params.astype(np.float64).copy()
        p[i] += h
        lp = C.loss_and_grad(p, img, R, t, TINY, round_bf16=False)[0]
        p[i] -= 2 * h
        lm = C.loss_and_grad(p, img, R, t, TINY, round_bf16=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - grad[i]) < 2e-4 * max(1.0, abs(fd)), (i, fd, grad[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], np.float32)
    r = C.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1.0) wins
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - (-3.140625)) < 1e-7 and r[4] == 0.0


def test_contrastive_gradient_matches_finite_differences():
    rng = np.random.default_rng(17)
    n, tau = 6, 0.2
    P = rng.standard_normal((n, 68))
    Rr = rng.standard_normal((n, 68))
    t = rng.standard_normal((n, 2))
    loss, gp, gr = C.contrastive(P, Rr, t, tau)
    h = 1e-6
    for X, g in ((P, gp), (Rr, gr)):
        for (i, j) in [(0, 0), (2, 17), (5, 63), (1, 64), (3, 67), (4, 65)]:
            Xp, Xm = X.copy(), X.copy()
            Xp[i, j] += h
            Xm[i, j] -= h
            args_p = (Xp, Rr) if X is P else (P, Xp)
            args_m = (Xm, Rr) if X is P else (P, Xm)
            fd = (C.contrastive(*args_p, t, tau)[0] - C.contrastive(*args_m, t, tau)[0]) / (2 * h)
            assert abs(fd - g[i, j]) < 1e-6 * max(1.0, abs(fd)), (i, j, fd, g[i, j])


def test_contrastive_prefers_matching_pairs():
    rng = np.random.default_rng(19)
    n = 8
    Z = rng.standard_normal((n, 68))
    t = np.zeros((n, 2))
    Z[:, 64:] = 0.0
    matched = C.contrastive(Z, Z, t, 0.1)[0]
    shuffled = C.contrastive(Z, Z[::-1].copy(), t, 0.1)[0]
    assert matched < shuffled


def test_output_gradient_backprop_matches_the_pose_loss_path():
    rng = np.random.default_rng(23)
    _, total = C.layout(TINY)
    params = rng.standard_normal(total) * 0.1
    img = rng.standard_normal((3, TINY[0][2], TINY[0][2]))
    R = _rot(rng, 3)
    t = rng.standard_normal((3, 2))
    loss, grad = C.loss_and_grad(params, img, R, t, TINY, round_bf16=False)
    acts = C.forward(params, img, TINY, round_bf16=False)
    _, g = C.head_loss(acts[-1], R, t)
    np.testing.assert_allclose(C.grad_from_output(params, img, g / 3, TINY, round_bf16=False),
                               grad, rtol=1e-12, atol=1e-14)
