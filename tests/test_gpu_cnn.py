"""The pose-proposal network's GPU kernels against the CPU oracle: the forward
pass (bf16 weights), the gradient of the pose loss for every parameter (FP32
weights, so the oracle's own finite-difference check carries over), and a
few Adam steps lowering the loss of a fixed batch."""
import numpy as np
import pytest
import torch

import tg3
from oracle import cnn_oracle as C

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _batch(n, seed):
    rng = np.random.default_rng(seed)
    img = rng.standard_normal((n, 64, 64)).astype(np.float32)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    t = rng.standard_normal((n, 2))
    return img, R, t


@pytest.fixture(scope="module")
def net():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    n = tg3.Cnn(0, seed=7)
    yield n
    n.close()


def test_forward_matches_oracle(net):
    img, R, t = _batch(3, 1)
    out = torch.empty((3, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    net.set_bf16(True)
    net.forward(torch.as_tensor(img).to(DEV), out)
    ref = C.forward(net.params(), img, round_bf16=True)[-1]
    got = out.cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-4, err


def test_gradient_matches_oracle(net):
    img, R, t = _batch(3, 2)
    net.set_bf16(False)
    net.zero_grads()
    loss = net.loss(torch.as_tensor(img).to(DEV), torch.as_tensor(R.reshape(3, 9)).to(DEV),
                    torch.as_tensor(t).to(DEV), grads=True)
    g = net.grads().astype(np.float64)
    net.set_bf16(True)
    ref_loss, ref = C.loss_and_grad(net.params(), img, R, t, round_bf16=False)
    assert abs(loss - ref_loss) < 1e-4 * max(1.0, abs(ref_loss)), (loss, ref_loss)
    lay, _ = C.layout()
    for li, (wo, ws, bo, co) in enumerate(lay):
        nw = int(np.prod(ws))
        for name, a, b in (("w", wo, wo + nw), ("b", bo, bo + co)):
            d = np.linalg.norm(g[a:b] - ref[a:b])
            r = np.linalg.norm(ref[a:b])
            assert d <= 2e-3 * r + 1e-7, (li, name, d, r)


def test_adam_lowers_the_loss(net):
    img, R, t = _batch(16, 3)
    im = torch.as_tensor(img).to(DEV)
    Rd = torch.as_tensor(R.reshape(16, 9)).to(DEV)
    td = torch.as_tensor(t).to(DEV)
    first = None
    for _ in range(30):
        net.zero_grads()
        v = net.loss(im, Rd, td, grads=True)
        first = v if first is None else first
        net.adam(1e-3)
    last = net.loss(im, Rd, td, grads=False)
    assert last < 0.8 * first, (first, last)


def test_proposals_follow_the_outputs():
    from tg3 import learned
    rng = np.random.default_rng(5)
    n, nR, nT = 6, 64, 9
    out = rng.standard_normal((n, tg3.Cnn.N_OUT)).astype(np.float32)
    od = torch.as_tensor(out).to(DEV)
    q = torch.empty((n, nR, 4), dtype=torch.float64, device=DEV)
    t = torch.empty((n, nT, 2), dtype=torch.float64, device=DEV)
    tg3.Cnn.propose(od, nR, nT, 11, q, t)
    torch.cuda.synchronize()
    q, t = q.cpu().numpy(), t.cpu().numpy()
    R, kap, w, mu, sd = learned.decode(out)
    centres = learned.mat_to_quat(R)
    assert np.allclose(np.abs((q[:, :8] * centres).sum(-1)), 1.0, atol=1e-9)
    assert np.allclose(np.linalg.norm(q, axis=-1), 1.0) and (q[..., 0] >= 0).all()
    assert np.allclose(t[:, 0], mu)
    # drawn rotations stay near their components (within a few 1/sqrt(kappa))
    ang = np.radians(learned.angle_deg(q[:, 8:, None, :], centres[:, None, :, :])).min(-1)
    assert (ang <= 6.0 / np.sqrt(kap.min(1))[:, None] + 1e-9).all()
