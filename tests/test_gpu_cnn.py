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


def test_contrastive_loss_matches_oracle(net):
    rng = np.random.default_rng(31)
    n, tau = 40, 0.1
    P = rng.standard_normal((n, tg3.Cnn.N_OUT)).astype(np.float32)
    Rr = rng.standard_normal((n, tg3.Cnn.N_OUT)).astype(np.float32)
    t = rng.standard_normal((n, 2))
    dP = torch.empty((n, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    dR = torch.empty_like(dP)
    loss = net.contrastive(torch.as_tensor(P).to(DEV), torch.as_tensor(Rr).to(DEV),
                           torch.as_tensor(t).to(DEV), tau, dP, dR)
    ref_loss, gp, gr = C.contrastive(P, Rr, t, tau)
    assert abs(loss - ref_loss) < 1e-5 * max(1.0, abs(ref_loss)), (loss, ref_loss)
    for got, ref in ((dP.cpu().numpy(), gp), (dR.cpu().numpy(), gr)):
        assert np.abs(got - ref).max() < 1e-4 * np.abs(ref).max()


def test_backward_from_outputs_matches_oracle(net):
    img, _, _ = _batch(3, 37)
    rng = np.random.default_rng(41)
    g_out = (rng.standard_normal((3, tg3.Cnn.N_OUT)) * 0.1).astype(np.float32)
    net.set_bf16(False)
    net.zero_grads()
    net.backward(torch.as_tensor(img).to(DEV), torch.as_tensor(g_out).to(DEV))
    g = net.grads().astype(np.float64)
    net.set_bf16(True)
    ref = C.grad_from_output(net.params(), img, g_out, round_bf16=False)
    lay, _ = C.layout()
    for li, (wo, ws, bo, co) in enumerate(lay):
        nw = int(np.prod(ws))
        for name, a, b in (("w", wo, wo + nw), ("b", bo, bo + co)):
            d = np.linalg.norm(g[a:b] - ref[a:b])
            r = np.linalg.norm(ref[a:b])
            assert d <= 2e-3 * r + 1e-7, (li, name, d, r)
    net.zero_grads()


def test_match_proposals_are_the_best_references():
    rng = np.random.default_rng(43)
    n, n_ref, n_rot, n_trans = 5, 300, 40, 9
    out = rng.standard_normal((n, tg3.Cnn.N_OUT)).astype(np.float32)
    ref = rng.standard_normal((n_ref, 64)).astype(np.float32)
    ref[7] = ref[3]                        # a tie: the lower index comes first
    ref /= np.linalg.norm(ref, axis=1, keepdims=True)
    rq = rng.standard_normal((n_ref, 4))
    rq /= np.linalg.norm(rq, axis=1, keepdims=True)
    od = torch.as_tensor(out).to(DEV)
    q = torch.empty((n, n_rot, 4), dtype=torch.float64, device=DEV)
    t = torch.empty((n, n_trans, 2), dtype=torch.float64, device=DEV)
    tg3.Cnn.match_propose(od, torch.as_tensor(ref).to(DEV), torch.as_tensor(rq).to(DEV), n_rot,
                          n_trans, 11, q, t)
    q2 = torch.empty((n, tg3.Cnn.N_OUT // 8 * 8, 4), dtype=torch.float64, device=DEV)
    t2 = torch.empty_like(t)
    tg3.Cnn.propose(od, q2.shape[1], n_trans, 11, q2, t2)
    z = torch.empty((n, 64), dtype=torch.float32, device=DEV)
    tg3.Cnn.embed(od, z)
    torch.cuda.synchronize()
    zp = z.cpu().numpy()
    np.testing.assert_allclose(zp, out[:, :64] / np.linalg.norm(out[:, :64], axis=1,
                                                                keepdims=True), rtol=1e-5)
    score = zp.astype(np.float64) @ ref.T.astype(np.float64)
    q = q.cpu().numpy()
    for l in range(n):
        sel = np.array([int(np.argmin(np.abs(rq - q[l, j]).sum(1))) for j in range(n_rot)])
        np.testing.assert_array_equal(rq[sel], q[l])
        # the selected set is the top n_rot by score (float32 scores: allow a
        # near-tie at the boundary), in descending order
        order = np.argsort(-score[l], kind="stable")
        assert len(set(sel) ^ set(order[:n_rot])) <= 2
        assert np.all(np.diff(score[l, sel]) <= 1e-5)
        if 3 in sel and 7 in sel:
            assert list(sel).index(3) < list(sel).index(7)
    np.testing.assert_array_equal(t.cpu().numpy(), t2.cpu().numpy())


def test_tensor_core_inference_matches_oracle(net):
    """tg3_cnn_infer (bf16 activations, implicit-GEMM convolutions on the
    tensor cores) against the float64 network with the same bf16 roundings;
    the accumulation order differs, so a hidden value near a bf16 rounding
    boundary may round the other way."""
    img, _, _ = _batch(37, 47)                  # not a multiple of the 128-pixel tile
    net.set_bf16(True)
    out = torch.empty((37, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    net.infer(torch.as_tensor(img).to(DEV), out)
    got = out.cpu().numpy().astype(np.float64)
    ref = C.forward(net.params(), img, round_bf16=True, round_act=True)[-1]
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-2, err
    cos = (got[:, :64] * ref[:, :64]).sum(1) / (np.linalg.norm(got[:, :64], axis=1) *
                                                np.linalg.norm(ref[:, :64], axis=1))
    assert cos.min() > 0.999, cos.min()
    # and close to the FP32-activation forward
    f32 = torch.empty_like(out)
    net.forward(torch.as_tensor(img).to(DEV), f32)
    ref32 = f32.cpu().numpy()
    assert np.abs(got - ref32).max() < 5e-2 * np.abs(ref32).max()


def test_inference_does_not_depend_on_the_batch(net):
    """2,100 images (two inference chunks of 2,048 and partial pixel tiles):
    every image's outputs are bit-identical to those of the same image in a
    batch of its own or of 5."""
    rng = np.random.default_rng(53)
    n = 2100
    img = torch.as_tensor(rng.standard_normal((n, 64, 64)).astype(np.float32)).to(DEV)
    net.set_bf16(True)
    out = torch.empty((n, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    net.infer(img, out)
    for i0, m in ((0, 1), (2047, 5), (2099, 1)):
        o2 = torch.empty((m, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
        net.infer(img[i0:i0 + m].contiguous(), o2)
        assert torch.equal(o2, out[i0:i0 + m])
