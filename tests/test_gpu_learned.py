"""What the trained proposal network gains over the method without it: after
a short training on particles of a few maps (the library's own kernels),
the rotations it proposes for new particles of those maps lie closer to the
true poses than those of the untrained network."""
import numpy as np
import pytest
import torch

import tg3
from tg3 import learned, synth

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def _nearest(net, ps, n_rot):
    n = len(ps.cls)
    out = torch.empty((n, tg3.Cnn.N_OUT), dtype=torch.float32, device=DEV)
    net.forward(ps.images, out)
    q = torch.empty((n, n_rot, 4), dtype=torch.float64, device=DEV)
    t = torch.empty((n, 1, 2), dtype=torch.float64, device=DEV)
    tg3.Cnn.propose(out, n_rot, 1, 3, q, t)
    torch.cuda.synchronize()
    return learned.angle_deg(q.cpu().numpy(), ps.quat_true[:, None, :]).min(1)


def test_training_brings_proposals_closer_to_the_truth():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    rng = np.random.default_rng(77)
    box, px = 128, 1.4
    maps = [synth.blob_map(rng, 120, (1.5, 3.0), px, 40.0) for _ in range(2)]
    rL = synth.config_rL(box, px)
    train = synth.particle_set(61, maps, np.arange(24000) % 2, box, px, 32, rL, 3.0, 1.0, device=DEV)
    test = synth.particle_set(62, maps, np.arange(400) % 2, box, px, 32, rL, 3.0, 1.0, device=DEV)
    net = tg3.Cnn(0, seed=3)
    try:
        before = _nearest(net, test, 64)
        R = torch.as_tensor(synth.quat_to_mat(train.quat_true).reshape(-1, 9)).to(DEV)
        t = torch.as_tensor(train.trans_true).to(DEV)
        losses = learned.train(net, train.images, R, t, 4, 256, 2e-3, seed=1)
        after = _nearest(net, test, 64)
    finally:
        net.close()
    assert losses[-1] < losses[0]
    # the trained proposals: nearer the truth for the median particle, and
    # within 15 degrees for clearly more particles than before
    assert np.median(after) < 0.8 * np.median(before), (np.median(before), np.median(after))
    assert np.mean(after < 15) > np.mean(before < 15) + 0.05, (np.mean(before < 15), np.mean(after < 15))
